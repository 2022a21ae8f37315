"""ctypes binding of libfe_gb300.so (the C-ABI in include/fe_gb300.h).

The library is built in-tree by ``pyoomph_gb300.build``.  There is no
fallback: if the library is missing or a call fails, an exception says so.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

(FE_OK, FE_ERR_ARG, FE_ERR_CUDA, FE_ERR_COMPILE, FE_ERR_NOMEM, FE_ERR_STATE, FE_ERR_DEVICE, FE_ERR_NOGPU,
 FE_ERR_SOLVER) = range(9)
FE_ASSEMBLE_RESIDUAL, FE_ASSEMBLE_JACOBIAN, FE_ASSEMBLE_VALUES_FROM_DOFS = 1, 2, 4
FE_ASSEMBLE_MASS, FE_ASSEMBLE_DPARAM, FE_ASSEMBLE_HVP, FE_ASSEMBLE_ZERO_FILTER = 8, 16, 32, 64
FE_GATHER_SLOTS, FE_GATHER_TILES = 0, 1
FE_JAC_F64, FE_JAC_F32 = 0, 1

INCLUDE_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc")
CACHE_DIR = os.environ.get("PYOOMPH_GB300_CACHE",
                           os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "_build",
                                        "jit_cache"))

# every symbol include/fe_gb300.h declares
EXPORTS = ["fe_last_error", "fe_version", "fe_device_info", "fe_code_compile", "fe_code_destroy", "fe_code_build",
           "fe_problem_create", "fe_problem_destroy", "fe_problem_sizes", "fe_problem_pattern",
           "fe_problem_pattern_device", "fe_problem_set_values", "fe_problem_get_values",
           "fe_problem_set_params", "fe_assemble", "fe_assemble_host", "fe_residual_max", "fe_dof_update",
           "fe_problem_check", "fe_problem_launch_count", "fe_problem_set_timing", "fe_problem_stage_times",
           "fe_problem_pipeline_times", "fe_problem_set_pipeline_streams", "fe_pattern_host",
           "fe_residual_max_noalloc", "fe_residual_max_noalloc_limit", "fe_problem_element_buffers",
           "fe_problem_set_history", "fe_problem_get_history", "fe_problem_shift_history", "fe_problem_set_positions",
           "fe_problem_graph_capture", "fe_problem_graph_launch", "fe_problem_set_dparam",
           "fe_assemble_pipelined", "fe_csr_spmv", "fe_csr_diagonal", "fe_krylov_create", "fe_krylov_solve",
           "fe_krylov_matvec", "fe_krylov_info", "fe_krylov_destroy", "fe_problem_set_direction",
           "fe_problem_set_persistent", "fe_problem_set_zero_threshold", "fe_problem_filtered_pattern",
           "fe_problem_set_gather", "fe_problem_gather_lanes",
           "fe_problem_set_tensor_contraction", "fe_tc_contract", "fe_sa_aggregate",
           "fe_csr_update", "fe_sa_level_build", "fe_sa_level_info", "fe_sa_level_copy", "fe_sa_level_destroy",
           "fe_csr_block", "fe_csr_update_f32", "fe_gmres_cgs2_scratch", "fe_gmres_cgs2",
           "fe_gather_cast_f32", "fe_sub_mul_f32", "fe_scatter_cast_f64"]


def _header_stamp() -> str:
    """Hash of the device headers the generated sources include, so that the
    cubin cache (keyed by source text) never serves an image built against
    an older header."""
    import hashlib
    h = hashlib.sha1()
    for f in ("fe_device.cuh", "fe_abi.h", "fe_df64.cuh"):
        with open(os.path.join(INCLUDE_DIR, f), "rb") as fp:
            h.update(fp.read())
    return "// device headers " + h.hexdigest()[:16] + "\n"


class FeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[fe_gb300 error {code}] {msg}")
        self.code = code


class DomainDesc(ctypes.Structure):
    _fields_ = [
        ("code", ctypes.c_void_p),
        ("nnode_el", ctypes.c_int),
        ("nlocal", ctypes.c_int),
        ("n_elem", ctypes.c_int64),
        ("conn", ctypes.c_void_p),
        ("local_node", ctypes.c_void_p),
        ("local_val", ctypes.c_void_p),
        ("tables", ctypes.c_void_p),
        ("n_tables", ctypes.c_int64),
        ("elems_per_block", ctypes.c_int),
        ("threads_per_block", ctypes.c_int),
        ("smem_bytes", ctypes.c_int),
        ("replica_elems", ctypes.c_int64),
    ]


class ProblemDesc(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int),
        ("n_nodes", ctypes.c_int64),
        ("nval", ctypes.c_int),
        ("x", ctypes.c_void_p),
        ("eqn", ctypes.c_void_p),
        ("n_dof", ctypes.c_int64),
        ("n_domains", ctypes.c_int),
        ("domains", ctypes.POINTER(DomainDesc)),
        ("n_params", ctypes.c_int),
        ("params", ctypes.c_void_p),
        ("jac_precision", ctypes.c_int),
        ("params_stride", ctypes.c_int),
        ("n_history", ctypes.c_int),
        ("x0", ctypes.c_void_p),
        ("fused", ctypes.c_int),
        ("n_hang", ctypes.c_int64),
        ("hang_slot", ctypes.c_void_p),
        ("hang_ptr", ctypes.c_void_p),
        ("hang_master", ctypes.c_void_p),
        ("hang_weight", ctypes.c_void_p),
    ]


_lib = None
_lock = threading.Lock()


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) the native library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(_build.LIB):
            if not build_if_missing:
                raise FeError(FE_ERR_STATE, f"native library missing: {_build.LIB}")
            _build.build()
        L = ctypes.CDLL(_build.LIB)
        vp, i64, c_int, sz = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_size_t
        L.fe_last_error.restype = ctypes.c_char_p
        L.fe_version.restype = ctypes.c_char_p
        L.fe_device_info.argtypes = [vp] * 5
        L.fe_code_compile.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, vp,
                                      ctypes.c_char_p, sz]
        L.fe_code_build.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, vp,
                                    ctypes.c_char_p, sz]
        L.fe_code_destroy.argtypes = [vp]
        L.fe_code_destroy.restype = None
        L.fe_problem_create.argtypes = [ctypes.POINTER(ProblemDesc), vp]
        L.fe_problem_destroy.argtypes = [vp]
        L.fe_problem_destroy.restype = None
        L.fe_problem_sizes.argtypes = [vp, vp, vp]
        L.fe_problem_pattern.argtypes = [vp, vp, vp]
        L.fe_problem_pattern_device.argtypes = [vp, vp, vp]
        L.fe_problem_set_values.argtypes = [vp, vp]
        L.fe_problem_get_values.argtypes = [vp, vp]
        L.fe_problem_set_params.argtypes = [vp, vp]
        L.fe_assemble.argtypes = [vp, vp, vp, vp, c_int, vp]
        L.fe_assemble_host.argtypes = [vp, vp, vp, vp, c_int]
        L.fe_residual_max.argtypes = [vp, vp, i64, vp, vp]
        L.fe_dof_update.argtypes = [vp, vp, vp, i64, vp]
        L.fe_problem_check.argtypes = [vp]
        L.fe_problem_launch_count.argtypes = [vp, c_int]
        L.fe_problem_set_timing.argtypes = [vp, c_int]
        L.fe_problem_stage_times.argtypes = [vp, vp, vp]
        L.fe_problem_pipeline_times.argtypes = [vp, vp, c_int]
        L.fe_problem_set_pipeline_streams.argtypes = [vp, c_int]
        L.fe_pattern_host.argtypes = [ctypes.POINTER(ProblemDesc), vp, vp, vp]
        L.fe_residual_max_noalloc.argtypes = [vp, i64, vp, vp]
        L.fe_problem_element_buffers.argtypes = [vp, c_int, vp, vp]
        L.fe_problem_set_history.argtypes = [vp, c_int, vp]
        L.fe_problem_get_history.argtypes = [vp, c_int, vp]
        L.fe_problem_set_zero_threshold.argtypes = [vp, ctypes.c_double]
        L.fe_problem_set_gather.argtypes = [vp, c_int]
        L.fe_sa_level_build.argtypes = [ctypes.c_int64, vp, vp, vp, vp, ctypes.c_int64, ctypes.POINTER(vp)]
        L.fe_sa_level_info.argtypes = [vp, vp, vp, vp]
        L.fe_sa_level_copy.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.fe_sa_level_destroy.argtypes = [vp]
        L.fe_sa_level_destroy.restype = None
        L.fe_csr_block.argtypes = [ctypes.c_int64, vp, vp, vp, c_int, c_int, vp, vp, vp, vp]
        L.fe_csr_update_f32.argtypes = [vp, vp, vp, vp, vp, vp, vp, ctypes.c_float, vp, ctypes.c_int64,
                                        ctypes.c_int64, vp]
        L.fe_gmres_cgs2_scratch.argtypes = [ctypes.c_int64, c_int]
        L.fe_gmres_cgs2_scratch.restype = ctypes.c_int64
        L.fe_gmres_cgs2.argtypes = [vp, ctypes.c_int64, ctypes.c_int64, c_int, vp, vp, vp, vp]
        L.fe_gather_cast_f32.argtypes = [vp, vp, ctypes.c_int64, vp, vp, vp]
        L.fe_sub_mul_f32.argtypes = [vp, vp, vp, vp, vp, ctypes.c_int64, vp]
        L.fe_scatter_cast_f64.argtypes = [vp, vp, ctypes.c_int64, vp, vp]
        L.fe_problem_gather_lanes.argtypes = [vp]
        L.fe_problem_filtered_pattern.argtypes = [vp, vp, vp, vp, vp]
        L.fe_problem_set_tensor_contraction.argtypes = [vp, c_int, c_int, c_int, c_int, vp, c_int, vp, vp]
        L.fe_tc_contract.argtypes = [vp, vp, i64, c_int, c_int, c_int, vp, c_int, vp, vp, vp]
        L.fe_sa_aggregate.argtypes = [i64, vp, vp, vp, vp, ctypes.c_double, vp, vp]
        L.fe_csr_update.argtypes = [vp, vp, vp, vp, vp, vp, vp, ctypes.c_double, vp, i64, i64, vp]
        L.fe_problem_shift_history.argtypes = [vp]
        L.fe_problem_set_positions.argtypes = [vp, vp]
        L.fe_problem_graph_capture.argtypes = [vp, vp, vp, vp, c_int]
        L.fe_problem_graph_launch.argtypes = [vp, vp]
        L.fe_problem_set_dparam.argtypes = [vp, c_int]
        L.fe_assemble_pipelined.argtypes = [vp, vp, vp, vp, c_int, c_int, vp]
        L.fe_csr_spmv.argtypes = [vp, vp, vp, c_int, vp, vp, i64, i64, vp]
        L.fe_csr_diagonal.argtypes = [vp, vp, vp, c_int, vp, i64, vp]
        L.fe_krylov_create.argtypes = [vp, vp, vp, c_int, i64, i64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, vp]
        L.fe_krylov_solve.argtypes = [vp, vp, vp, ctypes.c_double, ctypes.c_double, i64, ctypes.c_int32, vp, vp, vp]
        L.fe_krylov_info.argtypes = [vp, vp, vp, vp]
        L.fe_krylov_matvec.argtypes = [vp, vp, vp, vp]
        L.fe_krylov_destroy.argtypes = [vp]
        L.fe_krylov_destroy.restype = None
        L.fe_problem_set_direction.argtypes = [vp, vp, vp]
        L.fe_problem_set_persistent.argtypes = [vp, c_int]
        L.fe_residual_max_noalloc_limit.restype = i64
        _lib = L
        return L


def check(rc: int) -> None:
    if rc != FE_OK:
        raise FeError(rc, load().fe_last_error().decode(errors="replace"))


def code_build(source: str, name: str, cache_dir: str = CACHE_DIR) -> int:
    """nvrtc-compile only (no GPU needed); returns the cubin size."""
    L = load()
    os.makedirs(cache_dir, exist_ok=True)
    n = ctypes.c_size_t()
    log = ctypes.create_string_buffer(1 << 16)
    source = _header_stamp() + source
    rc = L.fe_code_build(source.encode(), name.encode(), INCLUDE_DIR.encode(), cache_dir.encode(),
                         ctypes.byref(n), log, len(log))
    if rc:
        raise FeError(rc, L.fe_last_error().decode(errors="replace") + "\n" + log.value.decode(errors="replace"))
    return n.value


class Code:
    """A compiled, loaded element kernel (owns the CUmodule)."""

    def __init__(self, source: str, name: str, cache_dir: str = CACHE_DIR):
        L = load()
        os.makedirs(cache_dir, exist_ok=True)
        h = ctypes.c_void_p()
        log = ctypes.create_string_buffer(1 << 16)
        source = _header_stamp() + source
        rc = L.fe_code_compile(source.encode(), name.encode(), INCLUDE_DIR.encode(), cache_dir.encode(),
                               ctypes.byref(h), log, len(log))
        if rc:
            raise FeError(rc, L.fe_last_error().decode(errors="replace") + "\n" + log.value.decode(errors="replace"))
        self.handle = h
        self.name = name

    def __del__(self):
        try:
            if self.handle:
                load().fe_code_destroy(self.handle)
                self.handle = None
        except Exception:
            pass
