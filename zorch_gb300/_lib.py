"""ctypes binding of the C ABI in include/zc.h (libzc.so, built in-tree).

The library is the only compute path: there is no CPU or PyTorch fallback.
If libzc.so is missing and cannot be built, importing the package's compute
modules raises.
"""

from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "_build" / "libzc.so"

ZC_OK, ZC_BAD_SHAPE, ZC_NOT_POW2, ZC_OOB_INDEX, ZC_OOM = 0, 1, 2, 3, 4
ZC_TIMEOUT, ZC_CUDA_ERR, ZC_BAD_ARG, ZC_UNSUPPORTED = 5, 6, 7, 8
BABYBEAR, KOALABEAR = 0, 1
DUPLEX_WORDS = 34


class ZcError(RuntimeError):
    def __init__(self, status: int, msg: str) -> None:
        super().__init__(msg)
        self.status = status


class LdeJob(C.Structure):
    _fields_ = [("coeffs", C.c_void_p), ("out", C.c_void_p), ("batch", C.c_int64),
                ("log_k", C.c_int32), ("log_blowup", C.c_int32), ("shift_mont", C.c_uint32),
                ("tile_log", C.c_int32), ("bit_reversed", C.c_int32), ("radix_log", C.c_int32)]


class Leaves(C.Structure):
    """zc_leaves: leaf p = concat_q base[q*group_stride + p*group_len ...]."""

    _fields_ = [("base", C.c_void_p), ("num_leaves", C.c_int64), ("groups", C.c_int32),
                ("group_len", C.c_int32), ("group_stride", C.c_int64)]


class MerkleJob(C.Structure):
    _fields_ = [("leaves", Leaves), ("layers", C.c_void_p), ("top_log", C.c_int32),
                ("count", C.c_int32), ("leaf_stride", C.c_int64), ("layer_stride", C.c_int64)]


_lock = threading.Lock()
_lib: C.CDLL | None = None


def _declare(lib: C.CDLL) -> None:
    vp, i64, i32, u32, sz = C.c_void_p, C.c_int64, C.c_int32, C.c_uint32, C.c_size_t
    st = C.c_int
    sig = {
        "zc_status_str": (C.c_char_p, [st]),
        "zc_last_error": (C.c_char_p, []),
        "zc_version": (C.c_int, []),
        "zc_launch_count": (C.c_ulonglong, []),
        "zc_init": (st, [C.c_int]),
        "zc_to_mont": (st, [st, vp, vp, i64, vp]),
        "zc_host_device_ptr": (st, [vp, C.POINTER(vp)]),
        "zc_to_mont_from_host": (st, [st, vp, vp, i64, i32, vp]),
        "zc_from_mont": (st, [st, vp, vp, i64, vp]),
        "zc_scale": (st, [st, vp, vp, i64, u32, vp]),
        "zc_poseidon2_builtin": (st, [st, C.POINTER(vp)]),
        "zc_poseidon2_create": (st, [st, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, u32,
                                     C.POINTER(vp)]),
        "zc_poseidon2_destroy": (st, [vp]),
        "zc_poseidon2_permute": (st, [vp, vp, i64, vp]),
        "zc_poseidon2_permute_host": (st, [vp, vp, i64]),
        "zc_rs_encode_workspace_bytes": (sz, [i64, C.c_int, C.c_int]),
        "zc_rs_encode": (st, [st, vp, i64, C.c_int, C.c_int, u32, u32, vp, vp, sz, vp]),
        "zc_rs_encode_noalloc": (st, [st, vp, i64, C.c_int, C.c_int, u32, u32, vp, vp]),
        "zc_rs_encode_bitrev": (st, [st, vp, i64, C.c_int, C.c_int, u32, u32, vp, vp, sz, vp]),
        "zc_merkle_commit": (st, [vp, Leaves, vp, vp]),
        "zc_merkle_open": (st, [Leaves, vp, vp, i32, vp, vp, vp, vp]),
        "zc_merkle_open_reduced": (st, [Leaves, vp, vp, i32, i32, vp, vp, vp]),
        "zc_strided_merkle_commit": (st, [vp, Leaves, i32, vp, vp]),
        "zc_fri_fold": (st, [st, vp, i64, C.c_int, vp, C.c_int, u32, u32, vp, vp]),
        "zc_fri_fold_commit": (st, [vp, vp, i64, C.c_int, vp, C.c_int, u32, u32, vp, vp, vp]),
        "zc_fri_fold_bitrev": (st, [st, vp, i64, C.c_int, vp, C.c_int, u32, u32, vp, vp]),
        "zc_fri_fold_k": (st, [st, vp, i64, C.c_int, vp, C.c_int, C.c_int, u32, u32, vp, vp]),
        "zc_fri_fold_commit_bitrev": (st, [vp, vp, i64, C.c_int, vp, C.c_int, u32, u32, vp, vp,
                                           vp]),
        "zc_fri_fold_commit_hop": (st, [vp, vp, i64, C.c_int, vp, C.c_int, u32, u32, i32, vp, vp,
                                        vp, i32, vp, vp]),
        "zc_merkle_commit_hop": (st, [vp, Leaves, vp, vp, i32, vp, vp]),
        "zc_smcs_bind_root": (st, [vp, vp, u32, u32, vp, vp]),
        "zc_eq_expand_workspace_bytes": (sz, [i32]),
        "zc_eq_expand": (st, [st, vp, i32, vp, vp, sz, vp]),
        "zc_eval_mle_workspace_bytes": (sz, [i32, i32]),
        "zc_eval_mle": (st, [st, vp, i32, i32, vp, vp, vp, sz, vp]),
        "zc_rlc_columns_ex": (st, [st, vp, i64, i32, vp, i32, i32, i32, vp, vp]),
        "zc_rlc_values": (st, [st, vp, i32, vp, i32, i32, i32, vp, vp]),
        "zc_ef4_inv": (st, [st, vp, vp, i64, vp]),
        "zc_sumcheck_workspace_bytes": (sz, []),
        "zc_sumcheck_message": (st, [st, vp, i64, vp, vp, vp, vp, vp, sz, vp]),
        "zc_sumcheck_fold": (st, [st, vp, i64, vp, i32, vp, vp, vp, vp, vp, vp]),
        "zc_duplex_hop": (st, [vp, vp, vp, vp, vp, vp, vp, i64, i32, vp, vp, vp, vp, vp, vp, vp]),
        "zc_duplex_hop_host": (st, [vp, vp, vp, vp, vp, vp, vp, i64, i32, vp, vp, vp, vp, vp, vp]),
        "zc_duplex_step": (st, [vp, vp, vp, i64, i32, vp, vp, i64, vp]),
        "zc_duplex_grind": (st, [vp, vp, i32, vp, vp]),
        "zc_rlc_columns": (st, [st, vp, i64, i32, vp, vp, vp]),
        "zc_fill_uniform": (st, [st, vp, i64, C.c_uint64, vp]),
        "zc_fill_u32": (st, [vp, i64, u32, vp]),
        "zc_copy_rows": (st, [vp, i64, vp, i64, i64, i64, vp]),
        "zc_rs_encode_batch_workspace_bytes": (sz, [vp, i32]),
        "zc_rs_encode_batch": (st, [st, vp, i32, u32, vp, sz, vp]),
        "zc_merkle_commit_batch": (st, [vp, vp, i32, vp, sz, vp]),
        "zc_eval_poly_workspace_bytes": (sz, [i64]),
        "zc_eval_poly": (st, [st, vp, i64, vp, i32, vp, vp, sz, vp]),
        "zc_deep_quotient": (st, [st, vp, i64, vp, i32, vp, u32, u32, i32, vp, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def lib() -> C.CDLL:
    """The loaded library (built on first use when nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            from . import build as _build

            if _build.toolchain_available():
                _build.build(force=bool(os.environ.get("ZC_REBUILD")))  # no-op when up to date
            elif not _LIB_PATH.exists():
                raise ZcError(ZC_CUDA_ERR, f"{_LIB_PATH} is missing and nvcc is not available")
            handle = C.CDLL(str(_LIB_PATH))
            _declare(handle)
            _lib = handle
    return _lib


def check(status: int, what: str = "") -> None:
    if status == ZC_OK:
        return
    L = lib()
    msg = f"{what}: {L.zc_status_str(status).decode()}"
    detail = L.zc_last_error().decode()
    if detail:
        msg += f" ({detail})"
    if status in (ZC_BAD_SHAPE, ZC_NOT_POW2):
        raise ValueError(msg)
    if status == ZC_OOB_INDEX:
        raise IndexError(msg)
    if status == ZC_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise ZcError(status, msg)


def library_path() -> Path:
    return _LIB_PATH
