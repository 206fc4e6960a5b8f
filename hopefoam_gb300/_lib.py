"""ctypes binding of libdgcu.so (include/dgcu.h).  Fails loudly when the
library is missing: there is no CPU fallback."""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libdgcu.so")

DG_OK, DG_ERR_ARG, DG_ERR_CUDA, DG_ERR_TIMEOUT, DG_ERR_NOT_CONVERGED, DG_ERR_NONFINITE, DG_ERR_UNSUPPORTED, \
    DG_ERR_NOMEM = range(8)
ERR_NAMES = {0: "DG_OK", 1: "DG_ERR_ARG", 2: "DG_ERR_CUDA", 3: "DG_ERR_TIMEOUT", 4: "DG_ERR_NOT_CONVERGED",
             5: "DG_ERR_NONFINITE", 6: "DG_ERR_UNSUPPORTED", 7: "DG_ERR_NOMEM"}
DG_FLUX_LF, DG_FLUX_ROE = 0, 1
DG_PREC_FP64, DG_PREC_SPLIT = 0, 1
DG_PC_NONE, DG_PC_BLOCK_JACOBI, DG_PC_LEARNED, DG_PC_LEARNED_ONLY, DG_PC_MULTILEVEL = 0, 1, 2, 3, 4
DG_PC_LEARNED_MULTILEVEL = 5
DG_LPC_RELU, DG_LPC_LINEAR, DG_LPC_SCHWARZ, DG_LPC_SCHWARZ_MLP = 0, 1, 2, 3

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p
_fp = ctypes.POINTER(ctypes.c_float)


class MeshDesc(ctypes.Structure):
    _fields_ = [("K", ctypes.c_int32), ("EToV", _ip), ("VXY", _dp), ("EToE", _ip), ("EToF", _ip), ("ROT", _ip),
                ("BC", _ip)]


class Opts(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int32), ("cubature", _dp), ("n_cubature", ctypes.c_int32),
                ("gamma", ctypes.c_double), ("stream", _vp)]


class Info(ctypes.Structure):
    _fields_ = [("K", ctypes.c_int32), ("order", ctypes.c_int32), ("Np", ctypes.c_int32), ("Ng", ctypes.c_int32),
                ("Nfp", ctypes.c_int32), ("Nfq", ctypes.c_int32), ("n_bfaces", ctypes.c_int32), ("stream", _vp),
                ("device_bytes", ctypes.c_size_t)]


class BatchTuning(ctypes.Structure):
    _fields_ = [("concurrent", ctypes.c_int32), ("ms_sequential", ctypes.c_double), ("ms_concurrent", ctypes.c_double),
                ("ms_fused", ctypes.c_double)]


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("rel_residual", ctypes.c_double), ("ms", ctypes.c_double)]


class InsBdata(ctypes.Structure):
    _fields_ = [("u_value", _dp), ("u_gradient", _dp), ("p_value", _dp), ("p_neumann_extra", _dp),
                ("p_data_scale", ctypes.c_double), ("u_data_scale", ctypes.c_double)]


class InsStats(ctypes.Structure):
    _fields_ = [("iterations_p", ctypes.c_int32), ("iterations_u", ctypes.c_int32 * 2),
                ("rel_residual_p", ctypes.c_double), ("rel_residual_u", ctypes.c_double), ("ms", ctypes.c_double)]


# name -> (restype, argtypes); every symbol declared in include/dgcu.h
SIGNATURES = {
    "dg_ctx_create": (ctypes.c_int, [ctypes.POINTER(MeshDesc), ctypes.POINTER(Opts), ctypes.POINTER(_vp)]),
    "dg_ctx_destroy": (ctypes.c_int, [_vp]),
    "dg_get_info": (ctypes.c_int, [_vp, ctypes.POINTER(Info)]),
    "dg_last_error": (ctypes.c_char_p, [_vp]),
    "dg_upload_state": (ctypes.c_int, [_vp, _dp]),
    "dg_download_state": (ctypes.c_int, [_vp, _dp]),
    "dg_upload_state_device": (ctypes.c_int, [_vp, _vp]),
    "dg_download_state_device": (ctypes.c_int, [_vp, _vp]),
    "dg_set_boundary_traces": (ctypes.c_int, [_vp, _dp]),
    "dg_euler_rhs": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp]),
    "dg_euler_rhs_device": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp]),
    "dg_forward_euler_stage": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int, ctypes.c_int]),
    "dg_sync": (ctypes.c_int, [_vp]),
    "dg_lserk4_step": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "dg_ssprk2_step": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "dg_cfl_dt": (ctypes.c_int, [_vp, ctypes.c_double, _dp]),
    "dg_reference_operators": (ctypes.c_int, [ctypes.c_int, _dp, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "dg_ipdg_setup": (ctypes.c_int, [_vp, ctypes.c_double]),
    "dg_ipdg_apply": (ctypes.c_int, [_vp, _dp, _dp]),
    "dg_ipdg_apply_device": (ctypes.c_int, [_vp, _vp, _vp]),
    "dg_ipdg_set_boundary_types": (ctypes.c_int, [_vp, _ip]),
    "dg_ipdg_set_mass": (ctypes.c_int, [_vp, ctypes.c_double]),
    "dg_set_node_locations": (ctypes.c_int, [_vp, _dp, _dp]),
    "dg_set_boundary_kinds": (ctypes.c_int, [_vp, _ip, _ip]),
    "dg_limit": (ctypes.c_int, [_vp]),
    "dg_reflect_boundary_traces": (ctypes.c_int, [_vp]),
    "dg_limited_ssprk2_step": (ctypes.c_int, [_vp, ctypes.c_double, _dp, ctypes.c_int, ctypes.c_int]),
    "dg_ins_create": (ctypes.c_int, [ctypes.POINTER(MeshDesc), ctypes.POINTER(Opts), _ip, _ip, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, ctypes.POINTER(_vp)]),
    "dg_ins_destroy": (ctypes.c_int, [_vp]),
    "dg_ins_last_error": (ctypes.c_char_p, [_vp]),
    "dg_ins_set_state": (ctypes.c_int, [_vp, _dp, _dp]),
    "dg_ins_get_state": (ctypes.c_int, [_vp, _dp, _dp]),
    "dg_ins_set_precision": (ctypes.c_int, [_vp, ctypes.c_int]),
    "dg_ins_step": (ctypes.c_int, [_vp, ctypes.POINTER(InsBdata), ctypes.c_double, ctypes.c_int,
                                   ctypes.POINTER(InsStats)]),
    "dg_ins_operator": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(InsBdata), _dp, _dp]),
    "dg_pcg_solve": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(SolveStats)]),
    "dg_pcg_solve_device": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(SolveStats)]),
    "dg_euler_rhs_noalloc": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int]),
    "dg_lpc_setup": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_int, ctypes.c_int]),
    "dg_lpc_add_residual": (ctypes.c_int, [_vp, _dp]),
    "dg_lpc_set_slope": (ctypes.c_int, [_vp, ctypes.c_double]),
    "dg_lpc_set_coarse": (ctypes.c_int, [_vp, ctypes.c_int]),
    "dg_lpc_train": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_ulonglong, _dp, _dp]),
    "dg_lpc_loss": (ctypes.c_int, [_vp, _dp, _dp, _dp]),
    "dg_lpc_energy_gradients": (ctypes.c_int, [_vp, _dp, _fp, _fp, _dp]),
    "dg_lpc_get_weights": (ctypes.c_int, [_vp, _fp, _fp]),
    "dg_lpc_set_weights": (ctypes.c_int, [_vp, _fp, _fp]),
    "dg_lpc_gradients": (ctypes.c_int, [_vp, _fp, _fp, ctypes.c_int, _fp, _fp, _dp]),
    "dg_lpc_apply": (ctypes.c_int, [_vp, _dp, _dp]),
    "dg_set_element_dt": (ctypes.c_int, [_vp, _dp]),
    "dg_batch_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, ctypes.POINTER(_vp)]),
    "dg_batch_destroy": (ctypes.c_int, [_vp]),
    "dg_batch_last_error": (ctypes.c_char_p, [_vp]),
    "dg_batch_tune": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.POINTER(BatchTuning)]),
    "dg_batch_get_shape": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _ip, _ip]),
    "dg_batch_set_schedule": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "dg_batch_run": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp]),
}
DG_NOALLOC_MAX_VALUES = 524288

_lib = None


class DGError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__("%s%s" % (ERR_NAMES.get(code, str(code)), (": " + msg) if msg else ""))
        self.code = code


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libdgcu.so not built (%s): run __graft_entry__.build() or "
                               "python -m hopefoam_gb300.build" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def dptr(a):
    return a.ctypes.data_as(_dp)


def iptr(a):
    return a.ctypes.data_as(_ip)
