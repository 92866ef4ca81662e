"""ctypes loading of the in-tree native libraries.

The CUDA library is required: if lib/libttg.so is missing the import fails
loudly (there is no CPU fallback for any GPU entry point)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(_PKG, "lib")

c_i32, c_i64, c_dbl, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    if not a.flags["C_CONTIGUOUS"] and not a.flags["F_CONTIGUOUS"]:
        raise ValueError("array must be contiguous")
    return a.ctypes.data_as(ctypes.c_void_p)


_host = None
_ttg = None


def host():
    """Host operator-producer library (built on demand: it is plain C++)."""
    global _host
    if _host is None:
        path = os.path.join(LIBDIR, "libttg_host.so")
        if not os.path.exists(path):
            from . import build
            build.build_host()
        _host = ctypes.CDLL(path)
        for name in ("ttg_host_assemble_hloc", "ttg_host_assemble_cnloc",
                     "ttg_host_assemble_hloc_once", "ttg_host_assemble_hloc_pattern"):
            getattr(_host, name).restype = ctypes.c_int
        _host.ttg_host_free.restype = None
        _host.ttg_host_free.argtypes = [ctypes.c_void_p]
    return _host


class TtgOpInfo(ctypes.Structure):
    _fields_ = [("n", c_i64), ("nnz_h", c_i64), ("nnz_c", c_i64), ("nproj", c_i32),
                ("group_rows", c_i32), ("n_groups", c_i64), ("stored_cols", c_i64),
                ("fill", c_dbl), ("device_bytes", c_i64), ("launches", c_i64),
                ("n_tiles", c_i64), ("tile_slots", c_i64), ("tile_fill", c_dbl),
                ("umma_tiles", c_i64), ("umma_slots", c_i64),
                ("shifted_orth", c_i64)]


class TtgSched(ctypes.Structure):
    _fields_ = [("low", c_i32), ("high", c_i32), ("n_low", c_i32), ("return_prev", c_i32)]


# entry point -> argtypes (restype is ttg_status = int for all unless listed)
_SIGS = {
    "ttg_device_query": [c_vp, c_vp, c_vp],
    "ttg_op_create": [c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_i32, c_vp],
    "ttg_op_create_tucker": [c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_i32,
                             c_vp],
    "ttg_op_destroy": [c_vp],
    "ttg_op_set_rr_precision": [c_vp, c_i32],
    "ttg_op_info": [c_vp, c_vp],
    "ttg_op_sync": [c_vp],
    "ttg_op_record": [c_vp, c_i32],
    "ttg_op_elapsed_ms": [c_vp, c_i32, c_i32, c_vp],
    "ttg_op_kernel_timing": [c_vp, c_i32],
    "ttg_op_kernel_time": [c_vp, c_i32, c_vp, c_vp],
    "ttg_block_create": [c_vp, c_i32, c_vp],
    "ttg_block_destroy": [c_vp],
    "ttg_block_set": [c_vp, c_vp, c_i64],
    "ttg_block_get": [c_vp, c_vp, c_i64],
    "ttg_block_set_device": [c_vp, c_vp, c_i64],
    "ttg_block_get_device": [c_vp, c_vp, c_i64],
    "ttg_block_copy": [c_vp, c_vp],
    "ttg_cheb_filter": [c_vp, c_vp, c_i32, c_dbl, c_dbl, c_dbl, TtgSched],
    "ttg_apply_h": [c_vp, c_vp, c_vp],
    "ttg_gram": [c_vp, c_vp, c_vp, c_vp],
    "ttg_gram_noalloc": [c_vp, c_vp, c_i64, c_i32, c_i64, c_vp, c_vp],
    "ttg_chol_qr": [c_vp, c_vp],
    "ttg_syev": [c_vp, c_i32, c_vp, c_vp, c_vp],
    "ttg_rayleigh_ritz": [c_vp, c_vp, c_i32, c_vp, c_vp],
    "ttg_rotate": [c_vp, c_vp, c_vp],
    "ttg_lanczos_bounds": [c_vp, c_vp, c_i32, c_vp, c_vp],
    "ttg_chfsi_pass": [c_vp, c_vp, c_i32, c_dbl, c_dbl, c_dbl, TtgSched, c_i32, c_vp],
    "ttg_fermi": [c_vp, c_i32, c_vp, c_dbl, c_dbl, c_i32, c_vp, c_vp],
    "ttg_op_set_kinetic": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp],
    "ttg_op_update_potential": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp],
    "ttg_tucker_sthosvd": [c_vp, c_vp, c_vp, c_dbl, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp],
    "ttg_tucker_reconstruct": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp],
    "ttg_grid_lda": [c_vp, c_i64, c_vp, c_vp, c_i32, c_vp],
    "ttg_grid_integrate": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp],
    "ttg_grid_lincomb": [c_i32, c_vp, c_vp, c_i64, c_vp, c_i32, c_vp],
    "ttg_grid_cp_sum": [c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, c_vp],
    "ttg_grid_ion_potential": [c_i32, c_vp, c_vp, c_dbl, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp],
    "ttg_density": [c_vp, c_vp, c_vp, c_i32, c_i32, c_i32, c_i32, c_i32, c_i32, c_vp, c_vp,
                    c_vp, c_vp],
    "ttg_hartree": [c_i32, c_vp, c_vp, c_i32, c_i32, c_i32, c_vp, c_i32, c_i32, c_i32,
                    c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, c_i32, c_i32,
                    c_vp, c_vp, c_vp, c_vp, c_vp],
    "ttg_hartree_device": [c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                           c_vp, c_vp],
    "ttg_density_device": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i32],
    "ttg_op_update_potential_device": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp],
    "ttg_tc_gemm": [c_i64, c_i64, c_i64, c_vp, c_i64, c_vp, c_i64, c_i32, c_vp, c_i64, c_vp],
    "ttg_atom_descriptors": [c_i32, c_vp, c_i32, c_dbl, c_dbl, c_dbl, c_dbl, c_vp],
    "ttg_mlp_create": [c_i32, c_vp, c_vp],
    "ttg_mlp_set_params": [c_vp, c_vp],
    "ttg_mlp_get_params": [c_vp, c_vp],
    "ttg_mlp_forward": [c_vp, c_vp, c_i32, c_vp],
    "ttg_mlp_gradients": [c_vp, c_vp, c_vp, c_i32, c_vp, c_vp],
    "ttg_mlp_train": [c_vp, c_vp, c_vp, c_i32, c_i32, c_i32, ctypes.c_float, ctypes.c_float,
                      ctypes.c_uint64, c_vp],
    "ttg_hartree_energy": [c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                           c_vp, c_vp, c_vp, c_vp, c_vp],
}
_OTHER = {
    "ttg_version": ([], ctypes.c_char_p),
    "ttg_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "ttg_op_stream": ([c_vp], c_vp),
    "ttg_block_cols": ([c_vp], c_i32),
    "ttg_kernel_launches": ([], c_i64),
    "ttg_mlp_destroy": ([c_vp], None),
    "ttg_mlp_num_params": ([c_vp], c_i64),
}

EXPORTED = sorted(list(_SIGS) + list(_OTHER))


def ttg_path() -> str:
    return os.path.join(LIBDIR, "libttg.so")


def ttg():
    """The CUDA library.  Raises if it has not been built."""
    global _ttg
    if _ttg is None:
        path = ttg_path()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = ctypes.CDLL(path)
        for name, args in _SIGS.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        for name, (args, res) in _OTHER.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = res
        _ttg = lib
    return _ttg


STATUS = {0: "OK", 1: "BAD_ARG", 2: "BAD_CSR", 3: "OOM", 4: "NOT_SPD", 5: "NONFINITE",
          6: "TIMEOUT", 7: "CUDA_ERR", 8: "NO_DEVICE", 9: "NOT_CONVERGED"}


class TtgError(RuntimeError):
    def __init__(self, code: int, what: str):
        self.code = code
        self.status = STATUS.get(code, str(code))
        super().__init__(f"{what}: {self.status}")


def check(code: int, what: str) -> None:
    if code != 0:
        raise TtgError(code, what)
