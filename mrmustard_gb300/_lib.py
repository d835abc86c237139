"""ctypes binding of ``libmm_gb300.so`` (the C ABI declared in include/mm_gb300.h).

The library is the only compute path of this package: if it is missing, or no
CUDA device is present, every entry point raises.  There is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

from . import _build_ext

HEADER = Path(__file__).resolve().parent.parent / "include" / "mm_gb300.h"

MM_OK = 0
STATUS_NAMES = {
    1: "MM_ERR_INVALID_ARG",
    2: "MM_ERR_UNSUPPORTED",
    3: "MM_ERR_TOO_LARGE",
    4: "MM_ERR_CUDA",
    5: "MM_ERR_WAIT_TIMEOUT",
    6: "MM_ERR_WORKSPACE",
    7: "MM_ERR_NO_DEVICE",
}

P = ctypes.c_void_p
I32 = ctypes.c_int
I64 = ctypes.c_int64
U64 = ctypes.c_uint64
SZ = ctypes.c_size_t

# name -> (restype, argtypes)
SIGNATURES = {
    "mm_status_string": (ctypes.c_char_p, [I32]),
    "mm_max_modes": (I32, []),
    "mm_last_cuda_error": (ctypes.c_char_p, []),
    "mm_launch_count": (I64, []),
    "mm_workspace_init": (I32, [P, SZ, P]),
    "mm_workspace_status": (I32, [P, P, ctypes.POINTER(I32)]),
    "mm_hermite_workspace_bytes": (SZ, [I32, P, I64]),
    "mm_hermite_fwd": (I32, [I32, P, P, P, P, I32, P, P, SZ, P]),
    "mm_hermite_fwd_batched": (I32, [I64, I32, P, P, P, P, I32, P, P, SZ, P]),
    "mm_hermite_vjp": (I32, [I32, P, P, P, P, P, P, P, P, SZ, P]),
    "mm_hermite_vjp_batched": (I32, [I64, I32, P, P, P, P, P, P, P, P, SZ, P]),
    "mm_hermite_vjp_noalloc": (I32, [I32, P, P, P, P, P, P, P, P]),
    "mm_hermite_checkpoint_elems": (I64, [I32, P, I32]),
    "mm_hermite_checkpoint_save": (I32, [I32, P, I32, P, P, P]),
    "mm_hermite_vjp_checkpointed_workspace_bytes": (SZ, [I32, P, I32]),
    "mm_hermite_vjp_checkpointed": (I32, [I32, P, I32, P, P, P, P, P, P, P, P, P, SZ, P]),
    "mm_ragged_plan_create": (I32, [I64, P, P, ctypes.POINTER(P)]),
    "mm_ragged_plan_destroy": (None, [P]),
    "mm_ragged_plan_workspace_bytes": (SZ, [P]),
    "mm_ragged_plan_amplitudes": (I64, [P]),
    "mm_ragged_plan_offsets": (I32, [P, P, P, P]),
    "mm_ragged_plan_set_tuning": (I32, [P, I64, I64]),
    "mm_ragged_plan_set_team_size": (I32, [P, I32]),
    "mm_ragged_plan_upload": (I32, [P, P, SZ, P]),
    "mm_ragged_fwd": (I32, [P, P, P, P, I32, P, P, SZ, P]),
    "mm_ragged_fwd_copy_g": (I32, [P, P, P, P, I32, P, P, P, SZ, P]),
    "mm_ragged_plan_set_copy_split": (I32, [P, I32]),
    "mm_ragged_vjp": (I32, [P, P, P, P, P, P, P, P, SZ, P]),
    "mm_ragged_vjp_copy_g": (I32, [P, P, P, P, P, P, P, P, P, SZ, P]),
    "mm_hermite_fwd_host": (I32, [I32, P, P, P, P, I32, P, P]),
    "mm_hermite_vjp_host": (I32, [I32, P, P, P, P, P, P, P, P]),
    "mm_test_wait_timeout": (I32, [P, SZ, U64, P]),
    "mm_probe_dfma": (I32, [P, I32, I32, P]),
    "mm_probe_division": (I32, [I64, U64, P, P]),
    "mm_selftest": (I32, [P, SZ, P, ctypes.POINTER(I32)]),
    "mm_fock_gemm_workspace_bytes": (SZ, [I32, I64, I64, I64, I32]),
    "mm_fock_gemm": (I32, [I32, I64, I64, I64, P, P, P, I32, P, SZ, P]),
    "mm_autoshape_batched": (I32, [I64, I32, P, P, P, ctypes.c_double, I64, I64, P, P]),
    "mm_binomial_workspace_bytes": (SZ, [I32, P]),
    "mm_binomial": (I32, [I32, P, P, P, P, ctypes.c_double, I64, P, P, P, SZ, P]),
    "mm_diagonal_slots": (I64, [I32]),
    "mm_diagonal_workspace_bytes": (SZ, [I32, P, I64]),
    "mm_diagonal_amps": (I32, [I32, P, I64, P, P, P, P, P, SZ, P]),
    "mm_diagonal_jacobian": (I32, [I32, P, P, P, P, P, P, SZ, P]),
    "mm_diagonal_vjp": (I32, [I32, P, P, P, P, P, P, P, P, P]),
    "mm_fast_diagonal_workspace_bytes": (SZ, [I32, P, I64]),
    "mm_fast_diagonal": (I32, [I32, P, I64, P, P, P, I32, P, P, SZ, P]),
    "mm_leftover_slots": (I64, [I32]),
    "mm_leftover_workspace_bytes": (SZ, [I32, P]),
    "mm_leftover_amps": (I32, [I32, P, P, P, P, P, P, SZ, P]),
    "mm_leftover_jacobian": (I32, [I32, P, P, P, P, P, P, SZ, P]),
    "mm_leftover_vjp": (I32, [I32, P, P, P, P, P, P, P, P, P]),
    "mm_tensor_permute": (I32, [I32, P, P, I64, P, P, P]),
    "mm_tensor_sum_inner": (I32, [I64, I64, P, P, P]),
    "mm_zgemm_batched": (I32, [I64, I64, I64, I64, P, I64, P, I64, P, I64, P]),
}


class MMError(RuntimeError):
    """Error status returned by the GB300 library."""

    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        name = STATUS_NAMES.get(status, str(status))
        msg = f"{where}: {name}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


_lib = None


def header_symbols() -> list[str]:
    """Names of every function the public header declares."""
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^MM_API\s+[\w\s\*]+?\b(mm_\w+)\s*\(", text, flags=re.M)))


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the shared library and bind its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build_ext.LIB
    if not path.exists() or _build_ext._stale():
        if not build_if_missing:
            raise RuntimeError(f"GB300 library not built: {path}")
        _build_ext.build()
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, where: str) -> None:
    if status != MM_OK:
        lib = load()
        detail = ""
        if status == 4:
            detail = lib.mm_last_cuda_error().decode(errors="replace")
        if status == 1:
            raise ValueError(f"{where}: invalid argument")
        raise MMError(status, where, detail)
