"""ctypes binding of the C ABI declared in include/simkit_gb300.h.

The shared library is built in-tree (``__graft_entry__.build()`` or
``python -m simkit_gb300.build``) into ``simkit_gb300/_build/``.  Every
product entry point of the package goes through this binding; if the library
is missing the first call raises ``RuntimeError`` - there is no CPU
fallback.
"""

from __future__ import annotations

import ctypes

import numpy as np
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsimkit_gb300.so")

c_i32 = ctypes.c_int32
c_i64 = ctypes.c_int64
c_dbl = ctypes.c_double
c_vp = ctypes.c_void_p

SKG_OK = 0
SKG_ERR_ARG = -1
SKG_ERR_CUDA = -2
SKG_ERR_NOT_CONVERGED = -3
SKG_ERR_LINESEARCH = -4
SKG_ERR_NONFINITE = -5
SKG_ERR_TIMEOUT = -6
SKG_ERR_CAPACITY = -7

SKG_FP64 = 0
SKG_MIXED = 1

STATUS_NAMES = {
    SKG_OK: "ok", SKG_ERR_ARG: "invalid argument", SKG_ERR_CUDA: "CUDA error",
    SKG_ERR_NOT_CONVERGED: "not converged", SKG_ERR_LINESEARCH: "line search exhausted",
    SKG_ERR_NONFINITE: "non-finite value", SKG_ERR_TIMEOUT: "grid wait timed out",
    SKG_ERR_CAPACITY: "capacity exceeded",
}


class CoarseC(ctypes.Structure):
    _fields_ = [("n_agg", c_i32), ("n_cblocks", c_i32), ("mode", c_vp), ("cb_ptr", c_vp), ("cb_slot", c_vp),
                ("cb_rc", c_vp), ("n_inst", c_i32), ("max_np", c_i32), ("m_floats", c_i64), ("inst_agg", c_vp),
                ("agg_inst", c_vp), ("inst_moff", c_vp), ("colpack", c_vp)]


class TetMeshC(ctypes.Structure):
    _fields_ = [
        ("n_verts", c_i64), ("n_tets", c_i64), ("n_blocks", c_i64),
        ("tets", c_vp), ("dinv", c_vp), ("dinv32", c_vp), ("vol", c_vp), ("mu", c_vp), ("lam", c_vp),
        ("mat32", c_vp), ("bsr_rowptr", c_vp), ("bsr_col", c_vp), ("bsr_diag", c_vp), ("bsr_row", c_vp),
        ("hc_ptr", c_vp), ("hc_src", c_vp), ("v2t_ptr", c_vp), ("v2t", c_vp), ("material", c_i32),
        ("coarse", ctypes.POINTER(CoarseC)),
        ("n_upper", c_i64), ("up_slot", c_vp), ("up_mirror", c_vp), ("hcu_ptr", c_vp), ("hcu_src", c_vp),
    ]


class ContactPlaneC(ctypes.Structure):
    _fields_ = [("p", c_dbl * 3), ("n", c_dbl * 3), ("k", c_dbl)]


class NewtonRecordC(ctypes.Structure):
    _fields_ = [("capacity", c_i32), ("g", c_vp), ("dx", c_vp), ("alpha_h", c_vp), ("residual_h", c_vp),
                ("pcg_iters_h", c_vp)]


class BEParamsC(ctypes.Structure):
    _fields_ = [
        ("dt", c_dbl), ("tol", c_dbl), ("max_newton", c_i32), ("precision", c_i32), ("pcg_rtol", c_dbl),
        ("pcg_max_iter", c_i32), ("do_line_search", c_i32), ("ls_alpha", c_dbl), ("ls_beta", c_dbl),
        ("ls_max_iter", c_i32), ("pcg_mode", c_i32), ("ls_threshold", c_dbl), ("profile", c_i32),
        ("pcg_variant", c_i32), ("batch_min_cluster", c_i32), ("batch_vec_kb", c_i32), ("integrator", c_i32),
        ("n_planes", c_i32), ("contact_mass_weighted", c_i32), ("planes", ctypes.POINTER(ContactPlaneC)),
        ("coarse_refresh", c_i32), ("stop_rule", c_i32), ("record", ctypes.POINTER(NewtonRecordC)),
        ("ew_gamma", c_dbl), ("ew_alpha", c_dbl),
    ]


class BEStateC(ctypes.Structure):
    _fields_ = [("u", c_vp), ("u_curr", c_vp), ("u_prev", c_vp), ("mass", c_vp), ("f_ext", c_vp), ("pinned", c_vp),
                ("u_warm", c_vp), ("u_prev2", c_vp), ("u_prev3", c_vp), ("x_rest", c_vp)]


class StepInfoC(ctypes.Structure):
    _fields_ = [
        ("newton_iters", c_i32), ("pcg_iters", c_i32), ("ls_trials", c_i32), ("status", c_i32),
        ("residual0", c_dbl), ("residual", c_dbl), ("min_alpha", c_dbl), ("energy", c_dbl),
        ("launches", c_i32), ("warm_used", c_i32), ("t_hessian_ms", c_dbl), ("t_assemble_ms", c_dbl),
        ("t_pcg_ms", c_dbl), ("t_gradient_ms", c_dbl), ("t_energy_ms", c_dbl),
    ]


class BatchC(ctypes.Structure):
    _fields_ = [("n_inst", c_i32), ("max_rows", c_i32), ("inst_rows", c_vp), ("inst_tets", c_vp),
                ("vert_inst", c_vp), ("tet_inst", c_vp), ("order", c_vp)]


P = ctypes.POINTER
_SIGNATURES = {
    "skg_version": (c_i32, []),
    "skg_last_error": (c_i32, [ctypes.c_char_p, ctypes.c_size_t]),
    "skg_snh_energy_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_snh_gradient_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_snh_hessian_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_mmnh_energy_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_mmnh_gradient_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_mmnh_hessian_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_arap_energy_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_arap_gradient_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_arap_hessian_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_fcr_energy_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_fcr_gradient_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_fcr_hessian_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_le_energy_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_le_gradient_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_le_hessian_element_F": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "skg_psd_project": (c_i32, [c_vp, c_vp, c_i64, c_i32, c_i32, c_vp]),
    "skg_contact_plane_terms": (c_i32, [c_vp, c_i64, ctypes.POINTER(ContactPlaneC), c_vp, c_vp, c_vp, c_vp, c_vp,
                                        c_vp]),
    "skg_tet_setup": (c_i32, [c_vp, c_vp, c_i64, c_i64, c_vp, c_vp, c_vp]),
    "skg_tet_deformation_gradient": (c_i32, [c_vp, c_vp, c_vp, c_i64, c_vp, c_vp]),
    "skg_tet_gradient_scatter": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_i64, c_vp, c_vp]),
    "skg_pattern_build": (c_i32, [c_vp, c_i64, c_i64, P(c_i64), c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "skg_assembly_workspace_size": (c_i64, [P(TetMeshC), c_i32]),
    "skg_snh_energy_x": (c_i32, [P(TetMeshC), c_vp, P(c_dbl), c_vp, c_vp]),
    "skg_snh_gradient_x": (c_i32, [P(TetMeshC), c_vp, c_vp, c_vp, c_vp]),
    "skg_snh_hessian_x": (c_i32, [P(TetMeshC), c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp]),
    "skg_snh_energy_u": (c_i32, [P(TetMeshC), c_vp, c_vp, P(c_dbl), c_vp, c_vp]),
    "skg_snh_gradient_u": (c_i32, [P(TetMeshC), c_vp, c_vp, c_vp, c_vp, c_vp]),
    "skg_snh_hessian_u": (c_i32, [P(TetMeshC), c_vp, c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp]),
    "skg_be_workspace_size": (c_i64, [P(TetMeshC), c_i32]),
    "skg_be_step": (c_i32, [P(TetMeshC), P(BEParamsC), P(BEStateC), c_vp, P(StepInfoC), c_vp]),
    "skg_batch_workspace_size": (c_i64, [P(TetMeshC), P(BatchC), c_i32]),
    "skg_be_step_batched": (c_i32, [P(TetMeshC), P(BatchC), P(BEParamsC), P(BEStateC), c_vp, P(StepInfoC),
                                    P(StepInfoC), c_vp]),
    "skg_be_batch_plan_create": (c_i32, [P(TetMeshC), P(BatchC), P(BEParamsC), P(BEStateC), c_vp, P(c_vp)]),
    "skg_be_batch_plan_step": (c_i32, [c_vp, P(StepInfoC), P(StepInfoC), c_vp]),
    "skg_be_batch_plan_destroy": (c_i32, [c_vp]),
    "skg_be_plan_eligible": (c_i32, [P(TetMeshC), P(BEParamsC)]),
    "skg_be_plan_create": (c_i32, [P(TetMeshC), P(BEParamsC), P(BEStateC), c_vp, P(c_vp)]),
    "skg_be_plan_step": (c_i32, [c_vp, P(StepInfoC), c_vp]),
    "skg_be_plan_destroy": (c_i32, [c_vp]),
    "skg_pcg_workspace_size": (c_i64, [c_i64]),
    "skg_pcg_bsr64": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_dbl, c_i32, P(c_i32), c_vp, c_vp]),
    "skg_mlp_gemm": (c_i32, [c_vp, c_i64, c_i64, c_vp, c_i32, c_i64, c_i64, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp,
                             c_i32, c_i32, c_vp, c_vp]),
    "skg_mlp_gelu_backward": (c_i32, [c_vp, c_vp, c_i64, c_vp, c_vp]),
    "skg_mlp_transpose": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_vp, c_i32, c_vp]),
    "skg_mlp_reduce_splits": (c_i32, [c_vp, c_i32, c_i64, c_vp, c_vp]),
    "skg_mlp_colsum": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_vp, c_vp]),
    "skg_mlp_mse": (c_i32, [c_vp, c_i32, c_vp, c_i32, c_i32, c_vp, c_i32, c_vp, P(c_dbl), c_vp]),
    "skg_mlp_adam": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_i32, c_i32, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                             ctypes.c_float, c_i32, c_vp, c_i32, c_vp, c_i32, c_vp]),
    "skg_warmstart_features": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_dbl, c_i64, c_vp, c_vp, c_i32, c_vp,
                                       c_vp, c_vp, c_vp, c_vp]),
    "skg_warmstart_apply": (c_i32, [c_vp, c_vp, c_vp, c_i32, c_vp, c_dbl, c_i64, c_vp, c_vp]),
    "skg_warmstart_targets": (c_i32, [c_vp, c_vp, c_vp, c_dbl, c_i64, c_vp, c_vp]),
    "skg_pcg_noalloc_max_rows": (c_i64, []),
    "skg_pcg_bsr64_noalloc": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_dbl, c_i32, P(c_i32), c_vp]),
    "skg_wait_selftest_workspace_size": (c_i64, []),
    "skg_wait_selftest": (c_i32, [c_i32, c_i64, P(c_i32), c_vp, c_vp]),
}

_lock = threading.Lock()
_lib = None


def exported_symbols():
    """Names the header declares (used by the ABI tests)."""
    return list(_SIGNATURES)


def load():
    """Load the in-tree library; raise RuntimeError if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"simkit_gb300: CUDA library not built ({LIB_PATH} missing); run "
                    "`python -c 'import __graft_entry__ as g; g.build()'` first. There is no CPU fallback.")
            lib = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in _SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


class SimkitGpuError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    load().skg_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(status: int):
    if status != SKG_OK:
        msg = last_error()
        if status == SKG_ERR_ARG:
            raise ValueError(msg)
        raise SimkitGpuError(status, msg)
    return status


def contact_planes(planes):
    """ctypes array of contact planes from (k, p, n) triples (n is normalised)."""
    planes = list(planes or [])
    if len(planes) > 4:
        raise ValueError("at most 4 contact planes")
    arr = (ContactPlaneC * max(len(planes), 1))()
    for i, (k, p, n) in enumerate(planes):
        p = np.asarray(p, dtype=np.float64).reshape(3)
        n = np.asarray(n, dtype=np.float64).reshape(3)
        n = n / np.linalg.norm(n)
        arr[i].p[:] = list(p)
        arr[i].n[:] = list(n)
        arr[i].k = float(k)
    return arr, len(planes)
