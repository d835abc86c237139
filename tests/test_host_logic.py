"""Host-side logic of the facade (mirrors backend_manager.py:643-727 argument checks) and of
instance sharding.  These raise before any device work, so they run on the CPU."""

from __future__ import annotations

import numpy as np
import pytest

import mrmustard_gb300 as mm
from mrmustard_gb300 import shard


def test_out_too_small_raises():
    A, b, c = np.zeros((2, 2)), np.zeros(2), 1.0
    with pytest.raises(ValueError, match="too large for out.shape"):
        mm.hermite_renormalized(A, b, c, (4, 5), out=np.zeros((3, 5), complex))


def test_batch_mismatch_raises():
    A = np.zeros((3, 2, 2))
    b = np.zeros((2, 2))
    c = np.zeros(3)
    with pytest.raises(ValueError, match="b.shape"):
        mm.hermite_renormalized(A, b, c, (3, 3))
    with pytest.raises(ValueError, match="c.shape"):
        mm.hermite_renormalized(A, np.zeros((3, 2)), np.zeros(2), (3, 3))


def test_settings_context():
    assert mm.settings.STABLE_FOCK_CONVERSION is False
    with mm.settings(STABLE_FOCK_CONVERSION=True):
        assert mm.settings.STABLE_FOCK_CONVERSION is True
    assert mm.settings.STABLE_FOCK_CONVERSION is False


def test_shard_balances_cost():
    rng = np.random.default_rng(0)
    costs = rng.integers(1, 1000, 500)
    parts = shard.shard_instances(costs, 4)
    assert sorted(i for p in parts for i in p) == list(range(500))
    loads = [costs[p].sum() for p in parts]
    assert max(loads) - min(loads) <= costs.max()
    assert shard.shard_instances(costs, 1)[0] == list(range(500))


def test_einsum_subscript_parsing():
    """Host-side planning of the Fock einsum: explicit and implicit outputs (numpy's rule: labels
    seen once, sorted), errors for unknown/repeated output labels and ellipses."""
    from mrmustard_gb300.einsum import parse_subscripts

    assert parse_subscripts("ab,bc->ac", 2) == ([["a", "b"], ["b", "c"]], ["a", "c"])
    assert parse_subscripts("ba,cb", 2) == ([["b", "a"], ["c", "b"]], ["a", "c"])
    assert parse_subscripts("aa", 1) == ([["a", "a"]], [])
    assert parse_subscripts(" a b , b c -> c a ", 2) == ([["a", "b"], ["b", "c"]], ["c", "a"])
    import pytest

    with pytest.raises(ValueError):
        parse_subscripts("ab->ad", 1)
    with pytest.raises(ValueError):
        parse_subscripts("ab->aa", 1)
    with pytest.raises(ValueError):
        parse_subscripts("...a->a", 1)
    with pytest.raises(ValueError):
        parse_subscripts("ab,bc->ac", 3)


def test_diagonal_input_validation_raises_before_device_work():
    """The compactFock entry points check their inputs as inputValidation.py:25-58 and :61-100
    do (same exceptions and messages), before any device work."""
    A = np.eye(4, dtype=complex) * 0.1
    B = np.zeros(4, complex)
    with pytest.raises(ValueError, match="must be square"):
        mm.hermite_multidimensional_diagonal(np.zeros((4, 3), complex), B, 1.0, (3, 3))
    bad = A.copy()
    bad[0, 1] = np.nan
    with pytest.raises(ValueError, match="must not contain NaNs"):
        mm.hermite_multidimensional_diagonal(bad, B, 1.0, (3, 3))
    asym = A.copy()
    asym[0, 1] = 0.5
    with pytest.raises(ValueError, match="must be symmetric"):
        mm.hermite_multidimensional_diagonal(asym, B, 1.0, (3, 3))
    with pytest.raises(ValueError, match="unbactched or two dimensional"):
        mm.hermite_multidimensional_diagonal(A, np.zeros((4, 2, 2), complex), 1.0, (3, 3))
    with pytest.raises(ValueError, match="incompatible dimensions"):
        mm.hermite_multidimensional_diagonal(A, np.zeros(6, complex), 1.0, (3, 3))
    with pytest.raises(ValueError, match="array like of length M"):
        mm.hermite_multidimensional_diagonal(A, B, 1.0, 3)
    with pytest.raises(ValueError, match="A and cutoffs have incompatible"):
        mm.hermite_multidimensional_diagonal(A, B, 1.0, (3, 3, 3))
    with pytest.raises(TypeError, match="NumPy array"):
        mm.hermite_multidimensional_diagonal([[0.1, 0], [0, 0.1]], B, 1.0, (3,))


def test_leftover_input_validation_raises_before_device_work():
    """hermite_multidimensional_1leftoverMode's checks (inputValidation.py:103-119)."""
    A = np.eye(4, dtype=complex) * 0.1
    B = np.zeros(4, complex)
    with pytest.raises(ValueError, match="incompatible dimensions"):
        mm.hermite_multidimensional_1leftoverMode(A, np.zeros(6, complex), 1.0, (3, 3))
    with pytest.raises(ValueError, match="array like of length M"):
        mm.hermite_multidimensional_1leftoverMode(A, B, 1.0, 3)
    with pytest.raises(ValueError, match="A and cutoffs have incompatible"):
        mm.hermite_multidimensional_1leftoverMode(A, B, 1.0, (3, 3, 3))
    with pytest.raises(ValueError, match="greater than 1"):
        mm.hermite_multidimensional_1leftoverMode(np.eye(2, dtype=complex) * 0.1, np.zeros(2, complex), 1.0, (3,))
