"""ctypes binding of ``libfealpy_gb300.so`` (the C ABI in ``include/fealpy_gb300.h``).

This module is the only place that touches the shared library.  It loads the
in-tree build, declares every entry point's signature, maps status codes to the
exception types FEALPy raises (``ValueError`` for bad arguments,
``RuntimeError`` for everything found while running), and provides the small
amount of plumbing the host code needs: raw device pointers of torch tensors,
the current CUDA stream, and workspaces carved from torch's caching allocator.

There is no fallback: if the library is missing or no CUDA device is present,
every call raises.
"""
import ctypes
import os
import threading

import torch

from . import _build

_LOCK = threading.Lock()
_LIB = None

c_i32 = ctypes.c_int32
c_i64 = ctypes.c_int64
c_sz = ctypes.c_size_t
c_dbl = ctypes.c_double
c_vp = ctypes.c_void_p

FGB_F32 = 0
FGB_F64 = 1

FGB_CH_MEASURE = 0
FGB_CH_METRIC = 1
FGB_CH_GRAD = 16
FGB_MAX_CHANNELS = 16

STATUS_NAMES = {
    0: "ok", 1: "invalid argument", 2: "workspace missing or too small", 3: "index out of range",
    4: "contribution outside the CSR pattern", 5: "non-finite value", 6: "CG breakdown (matrix not SPD)",
    7: "CUDA error", 8: "size exceeds a fixed kernel limit",
}

PCG_REASONS = {0: "running", 1: "atol", 2: "rtol", 3: "maxit", 4: "zero rhs", 5: "breakdown", 6: "nonfinite",
               7: "stagnated"}


class AmgLevel(ctypes.Structure):
    """``fgb_amg_level`` (include/fealpy_gb300.h)."""
    _fields_ = [("n", c_i64), ("nnz", c_i64), ("indptr", c_vp), ("indices", c_vp), ("values", c_vp), ("dinv", c_vp),
                ("lmax", c_dbl), ("agg", c_vp), ("n_coarse", c_i64), ("member_ptr", c_vp), ("members", c_vp),
                ("values32", c_vp), ("dinv32", c_vp), ("sell", c_vp)]


class PcgInfo(ctypes.Structure):
    _fields_ = [("niter", c_i64), ("residual", c_dbl), ("b_norm", c_dbl), ("true_relres", c_dbl),
                ("reason", c_i32), ("n_updates", c_i32), ("launches", c_i64), ("kernel_ms", c_dbl),
                ("kernel_launches", c_i64), ("other_ms", c_dbl), ("extra_ms", c_dbl), ("graph", c_i32),
                ("reserved", c_i32)]


# name: (restype, [argtypes])
_SIGNATURES = {
    "fgb_status_string": (ctypes.c_char_p, [c_i32]),
    "fgb_abi_version": (c_i32, []),
    "fgb_scan_workspace_bytes": (c_sz, [c_i64]),
    "fgb_exclusive_scan_i32": (c_i32, [c_vp, c_i64, c_vp, c_vp, c_sz, c_vp]),
    "fgb_adjacency_workspace_bytes": (c_sz, [c_i64]),
    "fgb_adjacency_build": (c_i32, [c_i64, c_i32, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_pattern_workspace_bytes": (c_sz, [c_i64]),
    "fgb_pattern_count": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_pattern_fill": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_pattern_build": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_i32, c_i64, c_vp, c_vp, c_sz, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_pattern_compact": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_pattern_expand_blocks": (c_i32, [c_i64, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_cell_factors": (c_i32, [c_i32, c_i64, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp]),
    "fgb_assemble_workspace_bytes": (c_sz, [c_i64]),
    "fgb_assemble_scalar": (c_i32, [c_i32, c_i64, c_vp, c_vp, c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp,
                                    c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_pcg_multi_workspace_bytes": (c_sz, [c_i64, c_i32]),
    "fgb_pcg_multi_f64": (c_i32, [c_i64, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_dbl, c_dbl, c_i64, c_vp, c_vp,
                                  c_sz, c_vp]),
    "fgb_source_local": (c_i32, [c_i64, c_i32, c_i32, c_vp, c_i32, c_dbl, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_source_gather": (c_i32, [c_i64, c_vp, c_vp, c_i32, c_i32, c_vp, c_i32, c_dbl, c_vp, c_vp, c_vp, c_vp, c_i32,
                                  c_vp]),
    "fgb_csr_split_blocks": (c_i32, [c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp]),
    "fgb_local_matrices": (c_i32, [c_i32, c_i64, c_i32, c_i32, c_vp, c_vp, c_vp, c_i32, c_vp]),
    "fgb_local_elasticity_p1": (c_i32, [c_i32, c_i32, c_i64, c_vp, c_i32, c_vp, c_vp]),
    "fgb_assemble_scalar_acc": (c_i32, [c_i32, c_i64, c_vp, c_vp, c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp,
                                        c_vp, c_vp, c_i32, c_vp, c_vp, c_sz, c_vp]),
    "fgb_assemble_elasticity_p1": (c_i32, [c_i32, c_i32, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                           c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_dirichlet_count": (c_i32, [c_i32, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_dirichlet_fill": (c_i32, [c_i32, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_amg_setup_workspace_bytes": (c_sz, [c_i64]),
    "fgb_amg_aggregate": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_dbl, c_vp, ctypes.POINTER(c_i64), c_vp,
                                  ctypes.POINTER(c_dbl), c_vp, c_vp, c_sz, c_vp]),
    "fgb_amg_coarse_workspace_bytes": (c_sz, [c_i64, c_i64]),
    "fgb_amg_coarse_count": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, ctypes.POINTER(c_i64),
                                     c_vp, c_vp, c_sz, c_vp]),
    "fgb_amg_coarse_fill": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                    c_sz, c_vp]),
    "fgb_amg_workspace_bytes": (c_sz, [c_vp, c_i32]),
    "fgb_amg_vcycle": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_dbl, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_pcg_amg": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_dbl, c_vp, c_vp, c_dbl, c_dbl, c_i64, c_i32,
                            ctypes.POINTER(PcgInfo), c_vp, c_sz, c_vp]),
    "fgb_topology_workspace_bytes": (c_sz, [c_i64, c_i64]),
    "fgb_topology_count": (c_i32, [c_i64, c_i32, c_vp, c_i64, c_i32, c_i32, c_vp, ctypes.POINTER(c_i64), c_vp, c_vp,
                                   c_sz, c_vp]),
    "fgb_topology_fill": (c_i32, [c_i64, c_i32, c_vp, c_i64, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_sz,
                                  c_vp]),
    "fgb_cell_to_ipoint": (c_i32, [c_i64, c_i32, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_i64, c_vp, c_vp, c_vp,
                                   c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_cell_apply": (c_i32, [c_i32, c_i64, c_i32, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_csr_spmv": (c_i32, [c_i32, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, c_vp]),
    "fgb_csr_spmm_f64": (c_i32, [c_i64, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_residual_norm_workspace_bytes": (c_sz, []),
    "fgb_residual_norm": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_csr_diagonal": (c_i32, [c_i32, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_pcg_workspace_bytes": (c_sz, [c_i64]),
    "fgb_pcg_f64": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_dbl, c_dbl, c_i64, c_i32, c_i32, c_i32,
                            c_i32, c_vp, c_sz, ctypes.POINTER(PcgInfo), c_vp]),
    "fgb_pcg_f64_noalloc": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_dbl, c_dbl, c_i64, c_i32, c_i32,
                                    c_i32, ctypes.POINTER(PcgInfo), c_vp]),
    "fgb_pcg_mixed_workspace_bytes": (c_sz, [c_i64]),
    "fgb_pcg_mixed": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_dbl, c_dbl, c_i64, c_i32, c_i32,
                              c_i32, c_vp, c_sz, ctypes.POINTER(PcgInfo), c_vp]),
    "fgb_gather_sum": (c_i32, [c_i32, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_sell_slots": (c_i64, [c_i64]),
    "fgb_sell_workspace_bytes": (c_sz, [c_i64]),
    "fgb_sell_plan": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_sell_fill": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_sell_spmv": (c_i32, [c_i32, ctypes.c_void_p, c_vp, c_vp, c_vp]),
    "fgb_sell_d16_workspace_bytes": (c_sz, [c_i64]),
    "fgb_sell_renumber": (c_i32, [c_i64, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_csr_permute": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_sell_d16_indptr": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_sell_fill_d16": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_sell_d15_indptr": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_sell_fill_d15": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_permute": (c_i32, [c_i32, c_i64, c_vp, c_vp, c_vp, c_i32, c_vp]),
    "fgb_sell_b3_indptr": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "fgb_sell_fill_b3": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fgb_pcg_sell_workspace_bytes": (c_sz, [c_i64]),
    "fgb_pcg_sell_f64": (c_i32, [ctypes.c_void_p, c_vp, c_vp, c_vp, c_dbl, c_dbl, c_i64, c_i32, c_i32, c_i32, c_i32,
                                 c_vp, c_sz, ctypes.POINTER(PcgInfo), c_vp]),
    "fgb_sell_set_pipeline": (None, [c_i32]),
    "fgb_pcg_sell_mixed": (c_i32, [ctypes.c_void_p, c_vp, c_vp, c_vp, c_dbl, c_dbl, c_i64, c_i32, c_i32, c_i32,
                                   c_vp, c_sz, ctypes.POINTER(PcgInfo), c_vp]),
    "fgb_pcg_sell_mixed_ex": (c_i32, [ctypes.c_void_p, c_vp, c_vp, c_vp, c_dbl, c_dbl, c_i64, c_i32, c_i32, c_i32,
                                      c_i64, c_vp, c_sz, ctypes.POINTER(PcgInfo), c_vp]),
    "fgb_batch_bytes": (c_sz, [c_i32, c_i32, c_i32]),
    "fgb_batch_create": (c_i32, [c_i32, c_i32, c_i32, c_i32, c_vp, c_sz, ctypes.POINTER(c_vp)]),
    "fgb_batch_destroy": (c_i32, [c_vp]),
    "fgb_batch_set": (c_i32, [c_vp, c_i32, c_vp, c_i32, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp]),
    "fgb_batch_admit": (c_i32, [c_vp, c_i32, c_vp, c_vp, c_vp, c_dbl, c_vp]),
    "fgb_batch_run": (c_i32, [c_vp, c_i64, c_i32, c_vp, ctypes.POINTER(c_i32), ctypes.POINTER(c_i32), c_vp]),
    "fgb_batch_retire": (c_i32, [c_vp, c_i32, c_vp, c_vp]),
    "fgb_batch_spmv": (c_i32, [c_vp, c_vp, c_vp, c_vp]),
}


class BatchSystem(ctypes.Structure):
    """``fgb_batch_system`` (include/fealpy_gb300.h)."""
    _fields_ = [("n", c_i64), ("n_slices", c_i64)] + [(k, c_vp) for k in (
        "slice_ptr", "perm", "col", "val32", "val64", "dinv64", "b", "x", "r", "z", "p", "Ap", "y",
        "dinv32")] + [("fp64", c_i32), ("reserved", c_i32)]


class BatchState(ctypes.Structure):
    """``fgb_batch_state``."""
    _fields_ = [(k, c_dbl) for k in ("rz", "rz_prev", "rr", "alpha", "beta", "b_norm", "tol", "resid", "r_upd",
                                     "true_rel", "delta")] + [("niter", c_i64), ("maxit", c_i64)] + [
        (k, c_i32) for k in ("active", "done", "need_update", "n_updates", "reserved", "stall")] + [
        ("r_best", c_dbl), ("last_upd", c_i64), ("max_gap", c_i64)]


class BatchTile(ctypes.Structure):
    """``fgb_batch_tile``."""
    _fields_ = [("sys", c_i32), ("begin", c_i32), ("end", c_i32), ("reserved", c_i32)]


class SellDesc(ctypes.Structure):
    """``fgb_sell`` (include/fealpy_gb300.h)."""
    _fields_ = [("n", c_i64), ("n_slices", c_i64), ("slice_ptr", c_vp), ("perm", c_vp), ("col", c_vp),
                ("val64", c_vp), ("val32", c_vp), ("threads", c_i32), ("blocks", c_i32), ("col16", c_vp),
                ("col0", c_vp), ("node_triples", c_i32), ("col_long", c_i32)]


def library_path() -> str:
    return _build.LIB_PATH


def lib():
    """Load (building first if absent) and return the ctypes library handle."""
    global _LIB
    if _LIB is not None:
        return _LIB
    with _LOCK:
        if _LIB is None:
            path = library_path()
            if not os.path.exists(path):
                _build.build()
            handle = ctypes.CDLL(path)
            for name, (res, args) in _SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _LIB = handle
    return _LIB


def exported_symbols():
    return sorted(_SIGNATURES)


class FgbError(RuntimeError):
    def __init__(self, fn, code):
        self.code = code
        super().__init__(f"{fn} failed: {STATUS_NAMES.get(code, 'unknown')} (status {code})")


def check(fn_name, code):
    if code != 0:
        if code == 1:
            raise ValueError(f"{fn_name}: invalid argument (status 1)")
        raise FgbError(fn_name, code)


# Kernels each entry point launches per call (the solvers report theirs in
# fgb_pcg_info.launches).  Used to count this library's launches in a region.
KERNELS_PER_CALL = {
    "fgb_cell_factors": 1, "fgb_adjacency_build": 6, "fgb_pattern_count": 5, "fgb_pattern_fill": 2, "fgb_pattern_build": 5, "fgb_pattern_compact": 2,
    "fgb_pattern_expand_blocks": 2, "fgb_assemble_scalar": 2, "fgb_assemble_scalar_acc": 2, "fgb_local_matrices": 1, "fgb_csr_split_blocks": 2, "fgb_residual_norm": 2, "fgb_source_local": 1, "fgb_source_gather": 1, "fgb_local_elasticity_p1": 1, "fgb_assemble_elasticity_p1": 2,
    "fgb_dirichlet_count": 1, "fgb_exclusive_scan_i32": 3, "fgb_dirichlet_fill": 1, "fgb_csr_spmv": 1, "fgb_csr_spmm_f64": 1,
    "fgb_csr_diagonal": 1, "fgb_gather_sum": 1, "fgb_cell_apply": 1,
    "fgb_topology_count": 8, "fgb_topology_fill": 2, "fgb_cell_to_ipoint": 1, "fgb_sell_plan": 4, "fgb_sell_fill": 1, "fgb_sell_spmv": 1,
    "fgb_sell_renumber": 1, "fgb_csr_permute": 5, "fgb_sell_d16_indptr": 4, "fgb_sell_fill_d16": 1,
    "fgb_sell_d15_indptr": 4, "fgb_sell_fill_d15": 1, "fgb_permute": 1,
    "fgb_sell_b3_indptr": 4, "fgb_sell_fill_b3": 1,
}

_launches = [0]


def launch_count() -> int:
    """Kernels launched by this library in this process so far."""
    return _launches[0]


def add_launches(n: int):
    _launches[0] += int(n)


def call(name, *args):
    """Call an entry point and raise on a non-zero status."""
    code = getattr(lib(), name)(*args)
    check(name, code)
    _launches[0] += KERNELS_PER_CALL.get(name, 0)
    return code


# ---------------------------------------------------------------------------
# device plumbing
# ---------------------------------------------------------------------------
def require_cuda(t: torch.Tensor, name: str = "tensor"):
    if not isinstance(t, torch.Tensor) or t.device.type != "cuda":
        raise ValueError(f"{name} must be a CUDA tensor (fealpy_gb300 runs on the GPU only)")
    return t


def ptr(t):
    """Raw device pointer of a contiguous CUDA tensor (None -> NULL)."""
    if t is None:
        return None
    if t.device.type != "cuda":
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return ctypes.c_void_p(t.data_ptr())


def stream_ptr(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def dtype_code(dtype) -> int:
    if dtype == torch.float64:
        return FGB_F64
    if dtype == torch.float32:
        return FGB_F32
    raise ValueError(f"unsupported floating dtype {dtype}")


def workspace(nbytes: int, device) -> torch.Tensor:
    """Scratch buffer from torch's caching allocator (256-byte aligned)."""
    nbytes = max(int(nbytes), 256)
    return torch.empty(nbytes, dtype=torch.uint8, device=device)


def status_word(device) -> torch.Tensor:
    return torch.zeros(1, dtype=torch.int32, device=device)


def check_status_word(fn_name: str, st: torch.Tensor):
    code = int(st.item())
    if code != 0:
        raise FgbError(fn_name, code)
