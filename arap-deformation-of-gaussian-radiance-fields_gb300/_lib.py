"""ctypes binding of ``libarap_gb300.so`` (the C ABI in include/arap_gb300.h).

Loading never falls back to anything: if the library is missing the import of
the calling op fails with the reason.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libarap_gb300.so")

OK, NOT_CONVERGED, ENONFINITE, EBADINPUT, ETIMEOUT, ECUDA, ENOMEM, EUNSUPPORTED = range(8)
STATUS_NAMES = {0: "OK", 1: "NOT_CONVERGED", 2: "ENONFINITE", 3: "EBADINPUT",
                4: "ETIMEOUT", 5: "ECUDA", 6: "ENOMEM", 7: "EUNSUPPORTED"}
PRECISION_PLAIN, PRECISION_MIXED = 0, 1
KNN_MAX = 12
CENTER_SCRATCH_BYTES = 8 << 20  # ARAP_CENTER_SCRATCH_BYTES


class ArapError(RuntimeError):
    def __init__(self, fn, code):
        super().__init__("%s failed: %s (%d)" % (fn, STATUS_NAMES.get(code, "?"), code))
        self.code = code


class SolveConfig(C.Structure):
    _fields_ = [("w_rot", C.c_float), ("w_reg", C.c_float), ("w_con", C.c_float),
                ("weighting_factor", C.c_float), ("cons_on_center", C.c_int),
                ("max_iters", C.c_int), ("early_exit", C.c_int), ("precision", C.c_int),
                ("pcg_tol", C.c_float), ("pcg_max_iters", C.c_int), ("coarse_nodes", C.c_int),
                ("spin_limit", C.c_int), ("coarse_reuse", C.c_float)]


class GridInfo(C.Structure):
    _fields_ = [("min_xyz", C.c_float * 3), ("max_xyz", C.c_float * 3), ("step", C.c_float),
                ("interval", C.c_float), ("grid_num", C.c_int), ("n_valid", C.c_int),
                ("n_pairs", C.c_longlong)]


class SolveStats(C.Structure):
    _fields_ = [("status", C.c_int), ("gn_iterations", C.c_int), ("pcg_iterations", C.c_int),
                ("halvings", C.c_int), ("initial_energy", C.c_double), ("final_energy", C.c_double),
                ("n_free", C.c_int), ("n_static", C.c_int), ("n_rows", C.c_int),
                ("n_coarse", C.c_int), ("phase_ms", C.c_double * 9), ("resident", C.c_int),
                ("coarse_fallbacks", C.c_int), ("iteration_halvings", C.c_int * 64),
                ("coarse_inversions", C.c_int)]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["iteration_halvings"] = list(self.iteration_halvings)[:max(0, min(64, self.gn_iterations))]
        d["phase_ms"] = dict(zip(("setup", "gradient", "coarse", "pcg", "line_search", "coarse_invert",
                                 "pcg_spmv_work", "pcg_update_work", "pcg_coarse_work"), list(self.phase_ms)))
        return d


P = C.c_void_p
I = C.c_int
F = C.c_float
D = C.c_double

# name -> (restype, argtypes); every name here is declared in include/arap_gb300.h
SIGNATURES = {
    "arap_build_graph": (I, [P, I, I, P, P]),
    "arap_compute_weights": (I, [P, I, P, I, I, P, P, P, P]),
    "arap_compute_weights_ex": (I, [P, I, P, I, I, I, P, P, P, P]),
    "arap_knn_autotune": (I, [P, I, P, I, I, P, P, P]),
    "arap_solve_config_default": (None, [C.POINTER(SolveConfig)]),
    "arap_solver_create": (I, [C.POINTER(P), I, I, P, P, P, P, P, P, I, C.POINTER(SolveConfig), P]),
    "arap_solver_solve": (I, [P, P, P, P, P, C.POINTER(SolveStats), P]),
    "arap_solver_energy_grad": (I, [P, P, P, P, P, C.POINTER(D), P]),
    "arap_solver_status": (I, [P, P]),
    "arap_solver_free_count": (I, [P]),
    "arap_solver_free_ids": (I, [P, P]),
    "arap_solver_destroy": (None, [P]),
    "arap_solver_batch_create": (I, [P, P, I, F, P]),
    "arap_solver_batch_solve": (I, [P, P, P, P, P, P, P]),
    "arap_solver_batch_autotune": (I, [P, P, P, P, P, P, P]),
    "arap_solver_batch_ctas": (I, [P, P]),
    "arap_solver_batch_destroy": (None, [P]),
    "arap_node_table": (I, [I, P, P, P, P, P]),
    "arap_end_points": (I, [I, P, P, P, P, P, P]),
    "arap_skin_gaussians": (I, [I, I, P, P, P, P, P, P, P, P, P, P, P, I, P, P]),
    "arap_skin_plan_create": (I, [P, I, I, P, P, P]),
    "arap_skin_plan_info": (I, [P, P, P, P]),
    "arap_skin_plan_status": (I, [P, P]),
    "arap_skin_plan_destroy": (None, [P]),
    "arap_skin_gaussians_planned": (I, [P, P, P, P, P, P, P, P, P, P, P, P, I, P]),
    "arap_skin_gaussians_backward": (I, [I, I, P, P, P, P, P, P, P, P, P, P, P]),
    "arap_skin_gaussians_backward_planned": (I, [P, P, P, P, P, P, P, P, P, P, P]),
    "arap_node_quaternions": (I, [I, P, P, I, P, P]),
    "arap_skin_samples": (I, [I, I, P, P, P, P, P, P, P, P]),
    "arap_update_nodes": (I, [I, I, P, P, P, P, P, P]),
    "arap_static_mask": (I, [I, I, I, P, P, P, P]),
    "arap_aims_translate": (I, [P, P, I, F, F, F, P]),
    "arap_aims_twist": (I, [P, P, P, I, F, F, F, F, P]),
    "arap_aims_scale": (I, [P, P, P, I, F, P]),
    "arap_grid_build": (I, [C.POINTER(P), I, P, P, P, P, I, I, C.POINTER(GridInfo), P]),
    "arap_grid_arrays": (I, [P, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "arap_grid_status": (I, [P, P]),
    "arap_grid_center_order": (I, [P, I, P, P, P]),
    "arap_grid_center_order_noalloc": (I, [P, I, P, P, P]),
    "arap_ply_info": (I, [C.c_char_p, C.POINTER(C.c_int64), C.POINTER(I), C.POINTER(I)]),
    "arap_ply_load": (I, [C.c_char_p, C.c_int64, I, P, P, P, P, P, P, P, P]),
    "arap_ply_save": (I, [C.c_char_p, C.c_int64, P, P, P, P, P, P, P, P, C.POINTER(C.c_int64)]),
    "arap_grid_samples": (I, [P, P, P]),
    "arap_grid_ada_lpf": (I, [P, P, F, P, P]),
    "arap_grid_density": (I, [P, P, P, P, P, P, P, P, F, P, P, P]),
    "arap_stage2_loss_grad": (I, [P, P, P, P, P, P, P, P, F, P, P, P, F, P, P, P, P, P, C.POINTER(D), P]),
    "arap_stage2_adam": (I, [I, I, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P]),
    "arap_stage2_cell_flags": (I, [P, P, P, P, P]),
    "arap_grid_destroy": (None, [P]),
    "arap_render": (I, [I, P, P, P, P, P, F, I, P, P, P, F, F, I, I, P, P, P, P, P]),
    "arap_status_read": (I, [P, P]),
    "arap_version": (C.c_char_p, []),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load the library (building it first when absent and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build as _build  # noqa: WPS433
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(fn: str, code: int) -> int:
    if code not in (OK,):
        raise ArapError(fn, code)
    return code
