"""GB300-native Gaussian->Fock hot path of MrMustard.

The renormalised multidimensional Hermite recurrence (``vanilla`` / ``stable`` /
batched / VJP), the Fock contraction after it, the autoshape cutoffs before it, and the binomial
and diagonal (PNR / leftover-mode) strategies of the same recurrence, and the general Fock-space
einsum, computed by
hand-written sm_103a CUDA
kernels in ``libmm_gb300.so`` behind a C ABI (include/mm_gb300.h).  The Python layer mirrors
the reference's interface for this path; it has no CPU compute path.
"""

from __future__ import annotations

from ._build_ext import build as build_library
from .autograd import HermiteRenormalizedFn, hermite_renormalized_autograd
from .autoshape import autoshape_batched, autoshape_numba, ket_dm_triple
from .autotune import autotune
from .backend import BackendGB300
from .binomial import binomial, device_binomial, hermite_renormalized_binomial
from .diagonal import (
    fast_diagonal,
    grad_hermite_multidimensional_1leftoverMode,
    grad_hermite_multidimensional_diagonal,
    hermite_multidimensional_1leftoverMode,
    hermite_multidimensional_diagonal,
    hermite_renormalized_1leftoverMode,
    hermite_renormalized_diagonal,
    hermite_renormalized_1leftoverMode_autograd,
    hermite_renormalized_diagonal_autograd,
)
from .einsum import contract, einsum
from .fock import apply_unitary, fock_gemm
from .hermite import (
    device_fwd,
    device_vjp,
    checkpoint_elems,
    device_checkpoint_save,
    device_vjp_checkpointed,
    hermite_renormalized,
    hermite_renormalized_batched,
    stable,
    stable_numba,
    vanilla,
    vanilla_batch,
    vanilla_batch_numba,
    vanilla_batch_vjp,
    vanilla_batch_vjp_numba,
    vanilla_numba,
    vanilla_vjp,
    vanilla_vjp_numba,
)
from .ragged import RaggedBatch, plan_offsets
from .settings import settings

__version__ = "0.1.0"


def launch_count() -> int:
    """Kernel launches issued by libmm_gb300 in this process."""
    from . import _lib

    return int(_lib.load().mm_launch_count())


__all__ = [
    "BackendGB300",
    "HermiteRenormalizedFn",
    "RaggedBatch",
    "apply_unitary",
    "autoshape_batched",
    "autoshape_numba",
    "autotune",
    "binomial",
    "device_binomial",
    "contract",
    "einsum",
    "fast_diagonal",
    "grad_hermite_multidimensional_1leftoverMode",
    "grad_hermite_multidimensional_diagonal",
    "hermite_multidimensional_1leftoverMode",
    "hermite_renormalized_1leftoverMode_autograd",
    "hermite_multidimensional_diagonal",
    "hermite_renormalized_1leftoverMode",
    "hermite_renormalized_diagonal",
    "hermite_renormalized_diagonal_autograd",
    "build_library",
    "fock_gemm",
    "device_fwd",
    "device_vjp",
    "checkpoint_elems",
    "device_checkpoint_save",
    "device_vjp_checkpointed",
    "plan_offsets",
    "hermite_renormalized",
    "hermite_renormalized_autograd",
    "hermite_renormalized_batched",
    "hermite_renormalized_binomial",
    "ket_dm_triple",
    "launch_count",
    "settings",
    "stable",
    "stable_numba",
    "vanilla",
    "vanilla_batch",
    "vanilla_batch_numba",
    "vanilla_batch_vjp",
    "vanilla_batch_vjp_numba",
    "vanilla_numba",
    "vanilla_vjp",
    "vanilla_vjp_numba",
]
