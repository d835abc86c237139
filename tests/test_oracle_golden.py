"""Pin the CPU oracle (oracle/hermite_oracle.c) against outputs of the reference source itself.

tests/golden/hermite_golden.npz was produced by tests/golden/make_golden.py, which runs the
reference's own vanilla/{core,batch,gradients}.py and displacement.py unmodified.  Under
CPython the reference divides complex by real with numpy's reciprocal-multiply; with that
lowering selected the oracle must reproduce the fixtures bit for bit.  With numba's lowering
(true division, the default) it must agree to a few ulps.
"""

from __future__ import annotations

import numpy as np
import pytest
from scipy.special import eval_hermite, factorial

from conftest import golden_cases

import oracle


@pytest.fixture(autouse=True)
def _built():
    oracle.build()
    yield
    oracle.set_numpy_division(False)


def test_forward_bit_exact_numpy_division(golden):
    oracle.set_numpy_division(True)
    for n in golden_cases(golden, ("G", "G_stable")):
        sh = tuple(golden[f"{n}/shape"])
        A, b, c = golden[f"{n}/A"], golden[f"{n}/b"], golden[f"{n}/c"]
        assert np.array_equal(oracle.vanilla(sh, A, b, c), golden[f"{n}/G"]), n
        assert np.array_equal(oracle.stable(sh, A, b, c), golden[f"{n}/G_stable"]), n


def test_forward_numba_division_within_ulps(golden):
    for n in golden_cases(golden, ("G", "G_stable")):
        if n == "dgate":  # vanilla is unstable there (amplitudes ~1e7): only stable is meaningful
            continue
        sh = tuple(golden[f"{n}/shape"])
        A, b, c = golden[f"{n}/A"], golden[f"{n}/b"], golden[f"{n}/c"]
        assert oracle.rel_err(oracle.vanilla(sh, A, b, c), golden[f"{n}/G"]) < 1e-15, n
        assert oracle.rel_err(oracle.stable(sh, A, b, c), golden[f"{n}/G_stable"]) < 1e-15, n


def test_vjp_matches_reference(golden):
    for n in golden_cases(golden, ("dA",)):
        G, c, g = golden[f"{n}/G"], golden[f"{n}/c"], golden[f"{n}/dLdG"]
        dA, db, dc = oracle.vjp(G, c, g)
        # the fixture's sum(G*dLdG) is numpy's pairwise sum; the oracle's is numba's sequential one
        assert oracle.rel_err(dA, golden[f"{n}/dA"]) < 1e-14, n
        assert oracle.rel_err(db, golden[f"{n}/db"]) < 1e-14, n
        assert abs(dc - golden[f"{n}/dc"]) <= 1e-13 * max(1.0, abs(golden[f"{n}/dc"])), n


def test_batch_matches_reference(golden):
    sh = tuple(golden["batch/shape"])
    oracle.set_numpy_division(True)
    G = oracle.fwd_batch(sh, golden["batch/A"], golden["batch/b"], golden["batch/c"])
    assert np.array_equal(G, golden["batch/G"])
    Gs = oracle.fwd_batch(sh, golden["batch/A"], golden["batch/b"], golden["batch/c"], stable=True)
    assert np.array_equal(Gs, golden["batch/G_stable"])
    dA, db, dc = oracle.vjp_batch(golden["batch/G"], golden["batch/c"], golden["batch/dLdG"])
    assert oracle.rel_err(dA, golden["batch/dA"]) < 1e-14
    assert oracle.rel_err(db, golden["batch/db"]) < 1e-14
    assert oracle.rel_err(dc, golden["batch/dc"]) < 1e-14


def test_known_answer_hermite_1d(golden):
    """tests/test_math/test_special.py:23-36: 1-D values are He-polynomials / sqrt(n!)."""
    x = golden["kat1d/x"]
    expected = np.array([eval_hermite(i, x) / np.sqrt(factorial(i)) for i in range(5)]).T
    np.testing.assert_allclose(golden["kat1d/G"], expected, atol=1e-12)
    got = np.array([oracle.vanilla((5,), -2 * np.ones((1, 1)), 2 * np.array([x0]), 1.0) for x0 in x])
    np.testing.assert_allclose(got, expected, atol=1e-12)


def test_stable_dgate_matches_displacement(golden):
    """test_lattice_functions.py:141-152 at 60x60: stable == closed-form displacement."""
    G = oracle.stable((60, 60), golden["dgate/A"], golden["dgate/b"], golden["dgate/c"])
    assert np.allclose(G, golden["dgate/displacement"])


def test_ragged_oracle_equals_per_instance(golden):
    shapes = [tuple(golden[f"ragged{k}/shape"]) for k in range(7)]
    rh = oracle.RaggedHost(shapes)
    As = [golden[f"ragged{k}/A"] for k in range(7)]
    bs = [golden[f"ragged{k}/b"] for k in range(7)]
    cs = np.array([golden[f"ragged{k}/c"] for k in range(7)])
    G = oracle.fwd_ragged(rh, np.concatenate([a.ravel() for a in As]), np.concatenate(bs), cs)
    for k in range(7):
        o, n = rh.g_off[k], rh.sizes[k]
        assert np.array_equal(G[o:o + n].reshape(shapes[k]), oracle.vanilla(shapes[k], As[k], bs[k], cs[k]))
    dA, db, dc = oracle.vjp_ragged(rh, G, cs, G.conj())
    for k in range(7):
        rA, rb, rc = oracle.vjp(G[rh.g_off[k]:rh.g_off[k] + rh.sizes[k]].reshape(shapes[k]), cs[k],
                                G[rh.g_off[k]:rh.g_off[k] + rh.sizes[k]].conj().reshape(shapes[k]))
        D = len(shapes[k])
        assert np.array_equal(dA[rh.a_off[k]:rh.a_off[k] + D * D].reshape(D, D), rA)
        assert np.array_equal(db[rh.b_off[k]:rh.b_off[k] + D], rb)
        assert dc[k] == rc


# ---------------------------------------------------------------- autoshape
def test_autoshape_oracle_matches_reference(autoshape_golden):
    """The C restatement of autoshape_numba (autoshape.py:23-154) gives the reference source's
    shapes on every fixture case (tests/golden/make_autoshape_golden.py), with either lowering of
    the reference's complex/real division.  Includes the reference's own known answers:
    Coherent(alpha=1) -> (8,) (test_ket.py:98-100) and the vacuum -> (1,) (test_coherent.py:74-75)."""
    g = autoshape_golden
    assert tuple(g["coh1/shape"]) == (8,) and tuple(g["vac/shape"]) == (1,)
    try:
        for numpy_div in (True, False):
            oracle.set_numpy_division(numpy_div)
            for n in g["names"]:
                p, hi, lo = g[f"{n}/params"]
                got = oracle.autoshape(g[f"{n}/A"], g[f"{n}/b"], g[f"{n}/c"], p, int(hi), int(lo))
                assert np.array_equal(got, g[f"{n}/shape"]), (n, numpy_div, got, g[f"{n}/shape"])
    finally:
        oracle.set_numpy_division(False)


def test_autoshape_oracle_ragged_equals_single(autoshape_golden):
    g = autoshape_golden
    names = list(g["names"])
    shapes = oracle.autoshape_ragged([g[f"{n}/A"] for n in names], [g[f"{n}/b"] for n in names],
                                     [g[f"{n}/c"] for n in names], 0.999, 40, 2)
    for n, s in zip(names, shapes):
        assert np.array_equal(s, oracle.autoshape(g[f"{n}/A"], g[f"{n}/b"], g[f"{n}/c"], 0.999, 40, 2))


# ---------------------------------------------------------------- binomial
def test_binomial_oracle_matches_reference(binomial_golden):
    """The C restatement of binomial (strategies/binomial.py:30-70 with steps.vanilla_step) gives
    the reference source's tensors bit for bit under numpy's division lowering (and within 1e-15
    under numba's), the same stop weight (zero pattern), and the norm to 1e-15 (numpy's complex
    abs differs from hypot in the last bit)."""
    g = binomial_golden
    try:
        for numpy_div in (True, False):
            oracle.set_numpy_division(numpy_div)
            for n in g["names"]:
                l2, gc = g[f"{n}/params"]
                G, norm, _ = oracle.binomial(tuple(g[f"{n}/shape"]), g[f"{n}/A"], g[f"{n}/b"], g[f"{n}/c"], l2, int(gc))
                ref = g[f"{n}/G"]
                assert np.array_equal(G == 0, ref == 0), n
                if numpy_div:
                    assert np.array_equal(G, ref), n
                else:
                    assert np.abs(G - ref).max() <= 1e-15 * np.abs(ref).max(), n
                assert abs(norm - float(g[f"{n}/norm"])) <= 1e-15 * abs(float(g[f"{n}/norm"])), n
    finally:
        oracle.set_numpy_division(False)


def test_binomial_oracle_equals_vanilla_prefix(binomial_golden):
    """test_lattice_functions.py:122-138: binomial with local cutoffs (5, 5) equals the vanilla
    tensor's [:5, :5] block where it is filled."""
    g = binomial_golden
    A, b, c = g["vs_vanilla/A"], g["vs_vanilla/b"], g["vs_vanilla/c"]
    G, _, _ = oracle.binomial((5, 5), A, b, c, 0.9999, 12)
    V = oracle.vanilla((10, 10), A, b, c)[:5, :5]
    assert np.allclose(G, V)
