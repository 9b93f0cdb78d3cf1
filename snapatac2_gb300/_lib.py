"""Loader of ``libsnapgb300.so``, the C ABI declared in ``include/snapgb300.h``.

The library is built in-tree by ``snapatac2_gb300.build.build_library`` (nvcc,
``-gencode arch=compute_103a,code=sm_103a``).  There is no CPU fallback: every
compute entry point of this package goes through this library and raises
``RuntimeError`` when it is missing or when no CUDA device is present.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsnapgb300.so")

SG_OK = 0
SG_ERR_ARG = 1
SG_ERR_RANGE = 2
SG_ERR_CAP = 3
SG_ERR_CUDA = 4
SG_ERR_NUMERIC = 5
SG_ERR_TIMEOUT = 6
SG_ERR_PARSE = 7
SG_ERR_UNSORTED = 8
SG_ERR_CONVERT = 9
SG_ERR_COLLISION = 10

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int
_U32 = ctypes.c_uint32
_F64 = ctypes.c_double

# name -> (restype, argtypes); must match include/snapgb300.h
SIGNATURES: dict[str, tuple] = {
    "sg_version": (_I32, []),
    "sg_status_string": (ctypes.c_char_p, [_I32]),
    "sg_scan_scratch_bytes": (_I64, [_I64]),
    "sg_tile_scratch_bytes": (_I64, [_I64]),
    "sg_tile_plan": (_I32, [_P, _I64, _I64, _P, _P, _P, _P, _P, _I32, _U32, _I32, _I64, _I64, _P, _P,
                            _P, _P, _P]),
    "sg_tile_run": (_I32, [_P, _I64, _I64, _P, _P, _P, _P, _P, _I32, _U32, _I32, _I64, _I64, _P, _P,
                           _I64, _P, _P, _P, _P, _P]),
    "sg_tile_emit": (_I32, [_I64, _P, _P, _I64, _P, _P, _P, _I64, _P, _P]),
    "sg_col_counts": (_I32, [_I64, _I64, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sg_region_plan": (_I32, [_P, _I64, _I64, _P, _P, _P, _P, _I32, _P, _P, _P, _P, _P, _I64, _I32, _I64, _I64,
                              _P, _P, _P, _P, _P]),
    "sg_region_run": (_I32, [_P, _I64, _I64, _P, _P, _P, _P, _I32, _P, _P, _P, _P, _P, _I64, _I32, _I64, _I64,
                             _P, _P, _I64, _P, _P, _P, _P, _P]),
    "sg_frag_line_scratch_bytes": (_I64, [_I64]),
    "sg_frag_count_lines": (_I32, [_P, _I64, _P, _P, _P]),
    "sg_frag_index_lines": (_I32, [_P, _I64, _P, _I64, _P, _P]),
    "sg_frag_workspace_bytes": (_I64, [_I64, _I64]),
    "sg_frag_import": (_I32, [_P, _I64, _P, _I64, _P, _P, _P, _P, _P, _I32, ctypes.c_uint64, _P, _P, _I64, _I32,
                              ctypes.c_uint64, _I32, _I64, _I64, ctypes.c_uint64, _P, _I64, _P, _P]),
    "sg_frag_emit": (_I32, [_P, _I64, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sg_csr_row_ptr": (_I32, [_I64, _P, _P, _P, _P, _P]),
    "sg_csr_copy_rows": (_I32, [_I64, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sg_gather_bytes": (_I32, [_I64, _P, _P, _P, _P, _P, _P]),
    "sg_gene_max_scratch_bytes": (_I64, [_I64]),
    "sg_gene_max": (_I32, [_I64, _P, _P, _P, _P, _I64, _P, _I64, _P, _P, _P, _P, _P]),
    "sg_nystrom_rescale": (_I32, [_I64, _I32, _P, _P, _I64, _P, _P, _P]),
    "sg_radix_scratch_bytes": (_I64, [_I64]),
    "sg_radix_sort_u64": (_I32, [_I64, _P, _P, _P, _P, _I32, _I32, _P, _P, _P]),
    "sg_csr_select_cols": (_I32, [_I64, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sg_transpose_blocks": (_I32, []),
    "sg_transpose_work_bytes": (_I64, [_I64, _I64, _I32]),
    "sg_csr_transpose": (_I32, [_I64, _I64, _P, _P, _P, _I32, _P, _I64, _P, _P, _P, _P, _P, _P]),
    "sg_spectral_prepare": (_I32, [_I64, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                   _P, _P, _P, _P, _P, _P]),
    "sg_spmm": (_I32, [_I32, _I32, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _I32, _P]),
    "sg_spmm_variants": (_I32, []),
    "sg_spmm_ex": (_I32, [_I32, _I32, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _I32, _I32, _P]),
    "sg_proj_parts": (_I32, []),
    "sg_fill_random": (_I32, [_I32, _I64, ctypes.c_uint64, _P, _P]),
    "sg_block_proj": (_I32, [_I32, _I32, _I64, _P, _I64, _I32, _P, _P, _I32, _P, _P]),
    "sg_block_update": (_I32, [_I32, _I32, _I64, _P, _I64, _I32, _P, _P, _P]),
    "sg_block_cholqr": (_I32, [_I32, _I32, _I64, _P, _P, _I32, _P, _P, _P, _P, _P]),
    "sg_block_finish": (_I32, [_I32, _I32, _I64, _P, _P, _I64, _I32, _P, _P, _P, _P]),
    "sg_lanczos_hblock": (_I32, [_I32, _P, _I64, _I32, _P, _P, _P, _P, _P, _I32, _P]),
    "sg_knn_scratch_bytes": (_I64, [_I64, _I32, _I32, _I32]),
    "sg_knn": (_I32, [_P, _I64, _I32, _I32, _I32, _P, _P, _P, _I64, _P, _P]),
    "sg_knn_noalloc": (_I32, [_P, _I64, _I32, _I32, _I32, _P, _P, _P, _P]),
    "sg_bblock_proj": (_I32, [_I32, _I32, _I32, _I32, _P, _P, _P, _P, _P, _P, _I64, _I32, _P, _P, _P, _I64, _P]),
    "sg_bmask": (_I32, [_I64, _I32, _P, _P, _P, _P]),
    "sg_spmm_masked": (_I32, [_I32, _I32, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _I32, _I32, _P, _P]),
    "sg_spmm_staged_variants": (_I32, []),
    "sg_spmm_dyn": (_I32, [_I32, _I32, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _I32, _P, _P, _P]),
    "sg_spmm_ds_variants": (_I32, []),
    "sg_spmm_ds": (_I32, [_I32, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _I32, _P, _P, _P]),
    "sg_spmm_dyn_ordered": (_I32, [_I32, _I32, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _I32, _P, _P, _P]),
    "sg_row_order_positions": (_I64, [_I64]),
    "sg_row_order_scratch_bytes": (_I64, [_I64]),
    "sg_row_order": (_I32, [_I64, _P, _P, _P, _I64, _P]),
    "sg_ds_split": (_I32, [_I64, _P, _P, _P, _P]),
    "sg_idf_from_counts": (_I32, [_I64, _I64, _P, _P, _P, _P]),
    "sg_csr_row_norms": (_I32, [_I64, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sg_gather_ceiling": (_I32, [_I32, _I32, _I64, _P, _P, _P, _P]),
    "sg_staged_table_bytes": (_I64, [_I32, _I32, _I64, _I64]),
    "sg_staged_table": (_I32, [_I32, _I32, _I64, _I64, _P, _P, _P, _I64, _P]),
    "sg_spmm_staged": (_I32, [_I32, _I32, _I64, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _I32, _P, _P, _P]),
    "sg_bblock_update": (_I32, [_I32, _I32, _I64, _I32, _P, _P, _P, _I64, _I32, _P, _I64, _P, _P]),
    "sg_bblock_cholqr": (_I32, [_I32, _I32, _I64, _I32, _P, _P, _I32, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                _P]),
    "sg_blanczos_hblock": (_I32, [_I32, _I32, _P, _P, _I64, _I32, _P, _P, _I64, _P, _P, _P, _P]),
    "sg_bbasis_rotate": (_I32, [_I32, _I32, _I32, _P, _P, _P, _P, _I64, _I32, _P, _I64, _I64, _I32, _P, _I64, _P]),
    "sg_bidf": (_I32, [_I64, _P, _I32, _P, _P, _P, _P, _P]),
    "sg_adjoint_stage1": (_I32, [_I64, _I32, _P, _P, _P, _P, _I32, _P, _P, _P]),
    "sg_adjoint_stage2": (_I32, [_I64, _I32, _P, _I32, _P, _I32, _P, _P]),
    "sg_adjoint_stage3": (_I32, [_I64, _I32, _P, _P, _P, _P, _P, _I32, _P, _P]),
    "sg_adjoint_final": (_I32, [_I64, _I32, _P, _P, _I32, _P, _P, _P]),
    "sg_square_values": (_I32, [_I64, _P, _P, _P]),
    "sg_basis_rotate": (_I32, [_I32, _I32, _I64, _P, _I64, _I32, _P, _I64, _I32, _P, _I64, _P]),
    "sg_test_staged_fault": (_I32, [_I32, _I64]),
    "sg_csr_aggregate_count": (_I32, [_I64, _P, _P, _P, _P, _P, _P]),
    "sg_csr_aggregate_scratch_bytes": (_I64, [_I64, _I64]),
    "sg_csr_aggregate_run": (_I32, [_I32, _I64, _P, _P, _P, _P, _P, _I64, _P, _I64, _P, _I64, _P, _P, _P, _I64,
                                    _P, _P, _P]),
    "sg_sym_eig_work_bytes": (_I64, [_I32, _I32, _I32]),
    "sg_sym_eig": (_I32, [_I32, _P, _I64, _I32, _I32, _P, _P, _P, _I64, _P]),
    "sg_lanczos_work_bytes": (_I64, [_I32, _I32, _I32, _I64, _I64, _I32, _I32]),
    "sg_lanczos": (_I32, [_P, _I32, _I32, _I32, ctypes.c_uint64, _P, _P, _I64, _P, _P, _P, _P, _P, _P]),
}


class GramOp(ctypes.Structure):
    """``sg_gram_op``: the cosine operator of one dataset (device pointers)."""
    _fields_ = [("n", _I64), ("m", _I64), ("indptr", _P), ("indices", _P), ("values", _P), ("colptr", _P),
                ("rowidx", _P), ("cvalues", _P), ("w2", _P), ("a", _P), ("dinv", _P), ("w2_f32", _P),
                ("a_f32", _P), ("dinv_f32", _P), ("staged_table_t", _P), ("staged_table_x", _P),
                ("order_t", _P), ("order_t_positions", _I64)]


class LanczosOpts(ctypes.Structure):
    """``sg_lanczos_opts`` (zero / negative fields take the library defaults)."""
    _fields_ = [("basis", _I32), ("keep", _I32), ("tol_vec", _F64), ("tol_val", _F64),
                ("vec_positive_only", _I32), ("max_restarts", _I32), ("refine", _I32), ("variant_t", _I32),
                ("variant_x", _I32), ("refine_variant_t", _I32), ("refine_variant_x", _I32), ("time_spmm", _I32)]


class LanczosInfo(ctypes.Structure):
    """``sg_lanczos_info``."""
    _fields_ = [("block_matvecs", _I64), ("restarts", ctypes.c_int32), ("converged", ctypes.c_int32),
                ("basis", ctypes.c_int32), ("keep", ctypes.c_int32), ("max_residual", _F64),
                ("next_evals", _F64 * 4), ("seconds_cycles", _F64), ("seconds_ritz", _F64),
                ("seconds_restart", _F64), ("seconds_refine", _F64), ("spmm_ms_t", _F64), ("spmm_ms_x", _F64),
                ("spmm_launches", _I64), ("kernel_launches", _I64)]

# Kernels launched by one call of each entry point (launch accounting of the
# benchmark): e.g. sg_block_cholqr = projection partial + reduce + Cholesky +
# R⁻¹ application.
KERNELS_PER_CALL = {
    "sg_tile_plan": 4, "sg_tile_run": 5, "sg_tile_emit": 1, "sg_col_counts": 2, "sg_csr_select_cols": 5,
    "sg_csr_transpose": 8, "sg_spectral_prepare": 7, "sg_spmm": 1, "sg_spmm_ex": 1, "sg_spmm_masked": 1,
    "sg_spmm_staged": 1, "sg_spmm_dyn": 1, "sg_spmm_ds": 1, "sg_ds_split": 1, "sg_spmm_dyn_ordered": 1, "sg_row_order": 10, "sg_idf_from_counts": 3, "sg_csr_row_norms": 1, "sg_staged_table": 1, "sg_gather_ceiling": 1, "sg_block_proj": 2, "sg_block_update": 1, "sg_block_cholqr": 4, "sg_block_finish": 1,
    "sg_lanczos_hblock": 1, "sg_basis_rotate": 1, "sg_fill_random": 1, "sg_knn": 6, "sg_knn_noalloc": 6,
    "sg_bblock_proj": 2, "sg_bblock_update": 1, "sg_bblock_cholqr": 4, "sg_blanczos_hblock": 1,
    "sg_bbasis_rotate": 1, "sg_bidf": 3, "sg_bmask": 1,
    "sg_adjoint_stage1": 1, "sg_adjoint_stage2": 1, "sg_adjoint_stage3": 1, "sg_adjoint_final": 1,
    "sg_square_values": 1,
    "sg_frag_count_lines": 4, "sg_frag_index_lines": 1, "sg_region_plan": 4, "sg_region_run": 5,
    "sg_csr_row_ptr": 4, "sg_csr_copy_rows": 1, "sg_gather_bytes": 1, "sg_nystrom_rescale": 1,
    "sg_sym_eig": 7, "sg_csr_aggregate_count": 2, "sg_csr_aggregate_run": 14,
}

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


class SnapGB300Error(RuntimeError):
    """A status code other than SG_OK returned by the C ABI."""

    def __init__(self, code: int, what: str):
        self.code = code
        super().__init__(f"{what}: {status_string(code)} (status {code})")


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the shared library (no CUDA device needed to load it)."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                f"{p} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = ctypes.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def status_string(code: int) -> str:
    try:
        return load().sg_status_string(int(code)).decode()
    except Exception:  # noqa: BLE001 - used inside error paths
        return "unknown"


def lib() -> ctypes.CDLL:
    """The library, after checking that a CUDA device is usable."""
    if not torch.cuda.is_available():
        raise RuntimeError("snapatac2_gb300 needs a CUDA GPU (sm_103a); none is available")
    return load()


def check(code: int, what: str) -> None:
    if code != SG_OK:
        raise SnapGB300Error(int(code), what)


def ptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    return t.data_ptr()


class DeviceStatus:
    """Device-side status word + lowest offending index (see the C header)."""

    def __init__(self, device):
        self.buf = torch.zeros(2, dtype=torch.int64, device=device)
        self.buf[1] = -1  # 0xffff... as uint64: no offending entry yet

    @property
    def status_ptr(self) -> int:
        return self.buf.data_ptr()

    @property
    def bad_ptr(self) -> int:
        return self.buf.data_ptr() + 8

    def raise_if_error(self, what: str, index_name: str = "entry") -> None:
        v = self.buf.cpu().tolist()
        st = int(v[0]) & 0xFFFFFFFF
        if st != SG_OK:
            bad = v[1] & 0xFFFFFFFFFFFFFFFF
            extra = "" if bad == 0xFFFFFFFFFFFFFFFF else f" (first offending {index_name}: {bad})"
            err = SnapGB300Error(st, what + extra)
            err.bad_index = None if bad == 0xFFFFFFFFFFFFFFFF else bad
            raise err
