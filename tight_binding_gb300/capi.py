"""ctypes binding of libtbk's C ABI (``include/tbk.h``).

The library is built in-tree (``tight_binding_gb300/_build/libtbk.so``) by
``tight_binding_gb300.build``.  Loading fails loudly when it is missing: there
is no CPU fallback for any compute entry point.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libtbk.so"

TBK_OK = 0
TBK_ERR_INVALID = 1
TBK_ERR_CUDA = 2
TBK_ERR_NOMEM = 3
TBK_ERR_UNSUPPORTED = 4
TBK_ERR_TIMEOUT = 5
TBK_ERR_BUDGET = 6
TBK_PENDING = 7

PREC_FP64 = 0
PREC_MIXED = 1
PREC_DD = 2
FLAG_DOUBLING = 1 << 4
FLAG_DEVICE_PTRS = 1 << 5
FLAG_NO_L2_ZIGZAG = 1 << 6
FLAG_STAGED = 1 << 7
FLAG_TWO_STEP = 1 << 8
FLAG_NO_GRAPH = 1 << 9
FLAG_PERSISTENT = 1 << 10
FLAG_NO_CACHE = 1 << 11

BUILD_SPARSE = 0
BUILD_PERIODIC_BARE = 1
BUILD_BARE = 2

MU_CUDA_CORE, MU_TENSOR, MU_MIXED_RECURSION, MU_DD_RECURSION = 0, 1, 2, 4
MU_FUSED_OPS = 8
MU_BOTH_SIDES = 16
MU_FP64_BLOCKS = 32

KERNEL_DIRICHLET, KERNEL_FEJER, KERNEL_LORENTZ, KERNEL_JACKSON, KERNEL_LANCZOS, KERNEL_WANG_ZUNGER = range(6)

_i32, _i64, _u64, _d, _vp, _cp = C.c_int32, C.c_int64, C.c_uint64, C.c_double, C.c_void_p, C.c_char_p
_pi32, _pi64, _pd, _pu8 = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_uint8)


class ServerConfig(C.Structure):
    """tbk_server_config"""
    _fields_ = [("budget_gb", C.c_double), ("steps_per_round", C.c_int32), ("autotune", C.c_int32),
                ("max_resident", C.c_int32), ("result_arena_mb", C.c_int32), ("step_gb", C.c_double)]


class MomentsHeader(C.Structure):
    """tbk_moments_header (256 bytes)"""
    _fields_ = [("magic", C.c_char * 8), ("version", C.c_int32), ("kind", C.c_int32), ("rows", C.c_int32),
                ("cols", C.c_int32), ("is_complex", C.c_int32), ("R", C.c_int32), ("precision", C.c_int32),
                ("kernel", C.c_int32), ("seed", C.c_uint64), ("e_min", C.c_double), ("e_max", C.c_double),
                ("kernel_p0", C.c_double), ("kernel_p1", C.c_double), ("n_sites", C.c_int64),
                ("checksum", C.c_uint64), ("label", C.c_char * 160)]


MOMENTS_DOS, MOMENTS_MU_NM, MOMENTS_V_NM = 1, 2, 3


class Request(C.Structure):
    """tbk_request"""
    _fields_ = [("lattice", C.c_void_p), ("build_mode", C.c_int32), ("extend", C.c_int32 * 3),
                ("is_complex", C.c_int32), ("n_mom", C.c_int32), ("R", C.c_int32), ("precision", C.c_int32),
                ("seed", C.c_uint64), ("e_min", C.c_double), ("e_max", C.c_double),
                ("kind", C.c_int32), ("axis", C.c_int32 * 2), ("kernel", C.c_int32),
                ("kernel_p0", C.c_double), ("kernel_p1", C.c_double)]


REQ_DOS, REQ_KUBO_BASTIN, REQ_KUBO_GREENWOOD = 0, 1, 2


_pcfg, _preq = C.POINTER(ServerConfig), C.POINTER(Request)

# name -> (restype, argtypes); every function declared in include/tbk.h
SIGNATURES = {
    "tbk_last_error": (_cp, []),
    "tbk_version": (C.c_int, []),
    "tbk_device_count": (C.c_int, []),
    "tbk_cell_create": (C.c_int, [C.POINTER(_vp), _i32, _pd, _i32, C.POINTER(_cp), _pd]),
    "tbk_cell_copy": (C.c_int, [C.POINTER(_vp), _vp]),
    "tbk_cell_destroy": (None, [_vp]),
    "tbk_cell_add_hopping": (C.c_int, [_vp, _cp, _cp, _pi32, _d, _d]),
    "tbk_cell_add_hopping_nn": (C.c_int, [_vp, _cp, _i32, _d, _d]),
    "tbk_cell_atom_index": (C.c_int, [_vp, _cp, _pi32]),
    "tbk_cell_info": (C.c_int, [_vp, _pi32, _pi32, _pi32]),
    "tbk_cell_get_hoppings": (C.c_int, [_vp, _pi32, _pi32, _pi32, _pd]),
    "tbk_cell_get_geometry": (C.c_int, [_vp, _pd, _pd]),
    "tbk_cell_last_warnings": (C.c_int, [_vp, _pi32]),
    "tbk_lattice_create": (C.c_int, [C.POINTER(_vp), _vp, _pi32]),
    "tbk_lattice_destroy": (None, [_vp]),
    "tbk_lattice_total_number": (C.c_int, [_vp, _pi64]),
    "tbk_lattice_set_gauge_linear": (C.c_int, [_vp, _pd, _pd]),
    "tbk_lattice_set_gauge_sites": (C.c_int, [_vp, _pd]),
    "tbk_lattice_clear_gauge": (C.c_int, [_vp]),
    "tbk_lattice_set_scalar_sites": (C.c_int, [_vp, _pd]),
    "tbk_lattice_set_scalar_disorder": (C.c_int, [_vp, _d, _u64]),
    "tbk_lattice_set_removed": (C.c_int, [_vp, _pu8]),
    "tbk_lattice_remove_atoms": (C.c_int, [_vp, C.c_char_p, _pi32, _i64]),
    "tbk_lattice_remove_atoms_random": (C.c_int, [_vp, C.c_char_p, _i64, _u64]),
    "tbk_lattice_get_removed": (C.c_int, [_vp, _pu8]),
    "tbk_lattice_kept_number": (C.c_int, [_vp, _pi64]),
    "tbk_build_hamiltonian": (C.c_int, [C.POINTER(_vp), _vp, _i32, _pi32, _i32, _vp]),
    "tbk_build_position": (C.c_int, [C.POINTER(_vp), _vp, _i32, _vp]),
    "tbk_build_velocity_bond": (C.c_int, [C.POINTER(_vp), _vp, _i32, _pi32, _i32, _i32, C.c_double, _vp]),
    "tbk_sparse_from_csc": (C.c_int, [C.POINTER(_vp), _i32, _i32, _i64, _vp, _vp, _vp, _i32, _i32, _vp]),
    "tbk_sparse_info": (C.c_int, [_vp, _pi32, _pi32, _pi64, _pi32]),
    "tbk_sparse_row_classes": (C.c_int, [_vp, _pi32, _vp]),
    "tbk_sparse_download": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "tbk_sparse_destroy": (None, [_vp]),
    "tbk_sparse_rescale": (C.c_int, [C.POINTER(_vp), _vp, _d, _d, _vp]),
    "tbk_sparse_commutator": (C.c_int, [C.POINTER(_vp), _vp, _vp, _vp]),
    "tbk_spectral_range": (C.c_int, [_vp, _i32, _u64, _pd, _pd, _pd, _pd, _vp]),
    "tbk_cheb_expand": (C.c_int, [_vp, _i32, _vp, _i32, _vp, _vp, _i32, _vp]),
    "tbk_moments_save": (C.c_int, [_cp, _vp, _vp]),
    "tbk_moments_load_header": (C.c_int, [_cp, _vp]),
    "tbk_moments_load": (C.c_int, [_cp, _vp, _vp, _i64]),
    "tbk_expn_coef_alpha_seq": (C.c_int, [C.c_double, C.c_double, _i32, _vp]),
    "tbk_cheb_view_create": (C.c_int, [C.POINTER(_vp), _vp, _i32, _vp, _i32]),
    "tbk_cheb_view_next": (C.c_int, [_vp, _pi32, _vp, _vp]),
    "tbk_cheb_view_destroy": (None, [_vp]),
    "tbk_cheb_coef_delta": (C.c_int, [C.c_double, _i32, _vp]),
    "tbk_cheb_coef_evolution": (C.c_int, [C.c_double, C.c_double, C.c_double, _i32, _vp]),
    "tbk_cheb_evolution_terms": (C.c_int, [C.c_double, C.c_double, C.c_double, _pi32]),
    "tbk_cheb_braket_real": (C.c_int, [_i32, _i64, _vp, _vp, _vp, _i32, _vp, _vp, _i32, _i32, _vp]),
    "tbk_cheb_braket_complex": (C.c_int, [_i32, _i64, _vp, _vp, _vp, _i32, _vp, _vp, _i32, _i32, _vp]),
    "tbk_cheb_braket_release": (None, []),
    "tbk_kubo_release": (C.c_int, []),
    "tbk_set_wait_limit": (C.c_int, [_i64]),
    "tbk_kpm_create": (C.c_int, [C.POINTER(_vp), _vp, _i32, _i32]),
    "tbk_kpm_run": (C.c_int, [_vp, _i32, _vp, _vp, _vp, _vp]),
    "tbk_kpm_run_random": (C.c_int, [_vp, _i32, _u64, _vp, _vp]),
    "tbk_kpm_last_timing": (C.c_int, [_vp, _pd, _pi32, _pd]),
    "tbk_kpm_destroy": (None, [_vp]),
    "tbk_random_phase_kets": (C.c_int, [_i32, _i32, _u64, _vp]),
    "tbk_kernel_seq": (C.c_int, [_i32, _i32, _d, _d, _vp]),
    "tbk_green_imag_eval": (C.c_int, [_i32, _vp, _vp, _i32, _vp, _vp, _vp]),
    "tbk_green_imag_fft": (C.c_int, [_i32, _vp, _vp, _i32, _vp, _vp, _vp]),
    "tbk_dos_from_moments": (C.c_int, [_i32, _vp, _i32, _d, _d, _d, _i32, _vp, _vp, _vp]),
    "tbk_kubo_mu": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _i32, _i32, _u64, _vp, _i32, _d, _d, _i32, _d, _vp, _vp]),
    "tbk_kubo_last_timing": (C.c_int, [_pd, _pd, _pd, _pd, _pi32]),
    "tbk_mu_from_blocks": (C.c_int, [_i32, _i64, _vp, _vp, _i32, _vp, _vp]),
    "tbk_kubo_bastin_zeta": (C.c_int, [_i32, _vp, _i32, _vp, _d, _vp, _vp]),
    "tbk_kubo_greenwood_sigma": (C.c_int, [_i32, _vp, _i32, _vp, _d, _vp, _vp]),
    "tbk_kubo_bastin_integrate": (C.c_int, [_i32, _vp, _vp, _vp, _vp, _vp, _pi32]),
    "tbk_server_create": (C.c_int, [C.POINTER(_vp), _pcfg]),
    "tbk_server_destroy": (None, [_vp]),
    "tbk_server_submit": (C.c_int, [_vp, _preq, _pi64]),
    "tbk_server_poll": (C.c_int, [_vp, _i64, _i32, _vp, _vp]),
    "tbk_request_footprint": (C.c_int, [_preq, _pi64, _pi64]),
    "tbk_server_stats": (C.c_int, [_vp, _vp, _i32]),
    "tbk_server_tuning": (C.c_int, [_vp, _i32, _vp]),
    "tbk_cheb_moments_noalloc": (C.c_int, [_i32, _vp, _vp, _vp, _i32, _i32, _vp, _vp, _i32, _vp, _vp]),
}


class TbkError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"tbk error {code}: {msg}")
        self.code = code


_lib = None


def lib() -> C.CDLL:
    """The loaded libtbk (raises if it was not built)."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("TBK_LIBRARY", LIB_PATH))
        if not path.exists():
            raise ImportError(f"libtbk not built ({path} missing): run tight_binding_gb300.build")
        L = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != TBK_OK:
        raise TbkError(status, lib().tbk_last_error().decode(errors="replace"))


def ptr(a: np.ndarray | None) -> int | None:
    """Raw data pointer of a contiguous numpy array (None passes NULL)."""
    if a is None:
        return None
    if not a.flags["C_CONTIGUOUS"] and not a.flags["F_CONTIGUOUS"]:
        raise ValueError("array must be contiguous")
    return a.ctypes.data


def as_i32p(a: np.ndarray):
    return a.ctypes.data_as(_pi32)


def as_dp(a: np.ndarray):
    return a.ctypes.data_as(_pd)


def device_count() -> int:
    return int(lib().tbk_device_count())
