"""Backend object with the reference's plug-in interface for this path.

MrMustard dispatches ``math.hermite_renormalized`` by name to the active backend
(``BackendManager._apply``, mrmustard/math/backend_manager.py:89-116), which for the numpy
backend calls ``hermite_renormalized`` / ``hermite_renormalized_batched``
(mrmustard/math/backend_numpy.py:381-403), ``math.hermite_renormalized_binomial`` to
``hermite_renormalized_binomial`` (backend_numpy.py:405-421), and
``math.hermite_renormalized_diagonal`` / ``math.hermite_renormalized_1leftoverMode`` to the
methods of those names (backend_numpy.py:423-446), which use ``reorder_AB_bargmann``
(:367-375).  ``BackendGB300`` provides those methods with the same signatures; a maintainer
mixes it into the numpy backend so every other op keeps its numpy implementation.
"""

from __future__ import annotations

from .binomial import hermite_renormalized_binomial as _binomial
from .diagonal import hermite_renormalized_1leftoverMode as _leftover
from .diagonal import hermite_renormalized_diagonal as _diagonal
from .diagonal import reorder_AB_bargmann as _reorder
from .hermite import stable_numba, vanilla_batch_numba, vanilla_numba


class BackendGB300:
    name = "gb300"

    def hermite_renormalized(self, A, b, c, shape, stable=False, out=None):
        if stable:
            return stable_numba(tuple(shape), A, b, c, out)
        return vanilla_numba(tuple(shape), A, b, c, out)

    def hermite_renormalized_batched(self, A, b, c, shape, stable=False, out=None):
        return vanilla_batch_numba(tuple(shape), A, b, c, stable, out)

    def hermite_renormalized_binomial(self, A, B, C, shape, max_l2, global_cutoff):
        return _binomial(A, B, C, tuple(shape), max_l2, global_cutoff)

    def hermite_renormalized_diagonal(self, A, B, C, cutoffs, reorderedAB=True):
        return _diagonal(A, B, C, tuple(cutoffs), reorderedAB)

    def hermite_renormalized_1leftoverMode(self, A, b, c, output_cutoff, pnr_cutoffs, stable=False,
                                           reorderedAB=True):
        return _leftover(A, b, c, output_cutoff, tuple(pnr_cutoffs), stable, reorderedAB)

    def reorder_AB_bargmann(self, A, B):
        """(m0..m_{M-1}, m0'..) -> (m0, m0', m1, m1', ...) on A's rows and columns and B
        (backend_numpy.py:367-375)."""
        return _reorder(A, B)
