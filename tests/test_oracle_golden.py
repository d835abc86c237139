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

from conftest import ROOT, golden_cases

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


def test_many_modes_match_reference():
    """D = 5..8 (the largest mode counts of the GPU library, whose GPU tests compare with the
    oracle): the oracle's forward is bit-exact with the reference source under numpy's division
    lowering, its stable forward and VJP agree to the usual tolerances."""
    z = np.load(ROOT / "tests" / "golden" / "hermite_golden_many.npz")
    names = sorted({k.split("/")[0] for k in z.files})
    assert names == ["many5", "many6", "many7", "many8"]
    for n in names:
        sh = tuple(z[f"{n}/shape"])
        A, b, c = z[f"{n}/A"], z[f"{n}/b"], z[f"{n}/c"]
        oracle.set_numpy_division(True)
        assert np.array_equal(oracle.vanilla(sh, A, b, c), z[f"{n}/G"]), n
        assert np.array_equal(oracle.stable(sh, A, b, c), z[f"{n}/G_stable"]), n
        oracle.set_numpy_division(False)
        dA, db, dc = oracle.vjp(z[f"{n}/G"], c, z[f"{n}/dLdG"])
        assert oracle.rel_err(dA, z[f"{n}/dA"]) < 1e-14, n
        assert oracle.rel_err(db, z[f"{n}/db"]) < 1e-14, n
        assert abs(dc - z[f"{n}/dc"]) <= 1e-13 * max(1.0, abs(z[f"{n}/dc"])), n


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


def test_autoshape_oracle_matches_reference_many_modes():
    """M = 6..8 (squeezed vacua and coherent products, tests/golden/autoshape_golden_many.npz): the
    oracle gives the reference source's cutoffs; the GPU kernel is checked against the oracle there."""
    z = np.load(ROOT / "tests" / "golden" / "autoshape_golden_many.npz")
    assert sorted(str(n) for n in z["names"]) == ["coh6", "coh7", "coh8", "sq6", "sq7", "sq8"]
    try:
        for numpy_div in (True, False):
            oracle.set_numpy_division(numpy_div)
            for n in z["names"]:
                p, hi, lo = z[f"{n}/params"]
                got = oracle.autoshape(z[f"{n}/A"], z[f"{n}/b"], z[f"{n}/c"], p, int(hi), int(lo))
                assert np.array_equal(got, z[f"{n}/shape"]), (n, numpy_div, got, z[f"{n}/shape"])
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


def test_binomial_oracle_matches_reference_many_modes():
    """D = 5, 6, 8 (tests/golden/binomial_golden_many.npz: full fills and early stops at 30 %, 70 %
    and 95 % of the reachable norm): the oracle gives the reference source's tensors bit for bit
    under numpy's division lowering and its stop weights; the GPU is checked against the oracle."""
    z = np.load(ROOT / "tests" / "golden" / "binomial_golden_many.npz")
    assert len(z["names"]) == 15
    try:
        for numpy_div in (True, False):
            oracle.set_numpy_division(numpy_div)
            for n in z["names"]:
                l2, gc = z[f"{n}/params"]
                G, norm, _ = oracle.binomial(tuple(z[f"{n}/shape"]), z[f"{n}/A"], z[f"{n}/b"], z[f"{n}/c"], l2, int(gc))
                ref = z[f"{n}/G"]
                assert np.array_equal(G == 0, ref == 0), n
                if numpy_div:
                    assert np.array_equal(G, ref), n
                else:
                    assert np.abs(G - ref).max() <= 1e-15 * np.abs(ref).max(), n
                assert abs(norm - float(z[f"{n}/norm"])) <= 1e-15 * abs(float(z[f"{n}/norm"])), n
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


# ---------------------------------------------------------------- diagonal strategies
def _rel(x, ref):
    den = np.abs(ref).max()
    return float(np.abs(x - ref).max() / den) if den > 0 else float(np.abs(x - ref).max())


def test_diagonal_amps_oracle_matches_reference(diagonal_golden):
    """The C restatement of compactFock's diagonal amplitudes (diagonal_amps.py:17-248) gives the
    reference source's five arrays, with and without a batch axis on B, to 1e-14 relative (the
    reference's `A[i] @ G_in` is a BLAS dot with its own summation order), and the same zero
    pattern (the same elements written)."""
    from conftest import diagonal_cases

    g = diagonal_golden
    try:
        oracle.set_numpy_division(True)
        for n in diagonal_cases(g, "amps"):
            got = oracle.diagonal_amps(g[f"{n}/A"], g[f"{n}/B"], g[f"{n}/G0"], tuple(g[f"{n}/cutoffs"]))
            for name, x in zip(("arr0", "arr2", "arr1010", "arr1001", "arr1"), got):
                ref = g[f"{n}/{name}"]
                assert x.shape == ref.shape, (n, name)
                assert np.array_equal(x == 0, ref == 0), (n, name)
                assert _rel(x, ref) <= 1e-14, (n, name, _rel(x, ref))
    finally:
        oracle.set_numpy_division(False)


def test_diagonal_grad_oracle_matches_reference(diagonal_golden):
    """Jacobians of the diagonal amplitudes (diagonal_grad.py:17-378, inputValidation.py:82-100):
    dG0, dA (cutoffs + (2M, 2M)) and dB (cutoffs + (2M,)) to 1e-13 relative."""
    from conftest import diagonal_cases

    g = diagonal_golden
    try:
        oracle.set_numpy_division(True)
        for n in diagonal_cases(g, "grad"):
            got = oracle.diagonal_grad(g[f"{n}/A"], g[f"{n}/B"], g[f"{n}/G0"], tuple(g[f"{n}/cutoffs"]))
            for name, x in zip(("dG0", "dA", "dB"), got):
                ref = g[f"{n}/{name}"]
                assert x.shape == ref.shape, (n, name)
                assert _rel(x, ref) <= 1e-13, (n, name, _rel(x, ref))
    finally:
        oracle.set_numpy_division(False)


def test_diagonal_and_leftover_oracle_match_reference_many_modes():
    """M = 5, 6 (tests/golden/diagonal_golden_many.npz): the diagonal amplitudes and Jacobians, the
    leftover-mode blocks and Jacobians and fast_diagonal of the oracle against the reference source,
    with the tolerances of the M <= 4 tests; the GPU kernels are checked against the oracle there."""
    from conftest import diagonal_cases

    z = np.load(ROOT / "tests" / "golden" / "diagonal_golden_many.npz")
    assert sorted(str(z[f"{n}/kind"]) for n in z["names"]) == ["amps", "amps", "fd", "fd", "fd", "fd", "grad", "grad",
                                                                  "lo"]
    try:
        oracle.set_numpy_division(True)
        for n in diagonal_cases(z, "amps"):
            got = oracle.diagonal_amps(z[f"{n}/A"], z[f"{n}/B"], z[f"{n}/G0"], tuple(z[f"{n}/cutoffs"]))
            for name, x in zip(("arr0", "arr2", "arr1010", "arr1001", "arr1"), got):
                ref = z[f"{n}/{name}"]
                assert x.shape == ref.shape and np.array_equal(x == 0, ref == 0), (n, name)
                assert _rel(x, ref) <= 1e-14, (n, name, _rel(x, ref))
        for n in diagonal_cases(z, "grad"):
            got = oracle.diagonal_grad(z[f"{n}/A"], z[f"{n}/B"], z[f"{n}/G0"], tuple(z[f"{n}/cutoffs"]))
            for name, x in zip(("dG0", "dA", "dB"), got):
                assert _rel(x, z[f"{n}/{name}"]) <= 1e-13, (n, name)
        for n in diagonal_cases(z, "lo"):
            A, B, G0, cut = z[f"{n}/A"], z[f"{n}/B"], z[f"{n}/G0"], tuple(z[f"{n}/cutoffs"])
            for name, x in zip(("arr0", "arr2", "arr1010", "arr1001", "arr1"), oracle.leftover_amps(A, B, G0, cut)):
                ref = z[f"{n}/{name}"]
                assert x.shape == ref.shape and np.array_equal(x == 0, ref == 0), (n, name)
                assert _rel(x, ref) <= 1e-14, (n, name, _rel(x, ref))
            for name, x in zip(("dG0", "dA", "dB"), oracle.leftover_grad(A, B, G0, cut)):
                assert _rel(x, z[f"{n}/{name}"]) <= 1e-13, (n, name)
        for n in diagonal_cases(z, "fd"):  # fast_diagonal at L = 5, 6, vanilla and stable first block
            got = oracle.fast_diagonal(z[f"{n}/A"], z[f"{n}/b"], z[f"{n}/c"], int(z[f"{n}/oc"]),
                                       tuple(z[f"{n}/pnr"]), bool(z[f"{n}/stable"]))
            ref = z[f"{n}/out"]
            assert got.shape == ref.shape and np.array_equal(got == 0, ref == 0), n
            assert _rel(got, ref) <= 1e-14, (n, _rel(got, ref))
    finally:
        oracle.set_numpy_division(False)


def test_diagonal_amps_equal_vanilla_diagonal(diagonal_golden):
    """tests/test_math/test_compactFock.py:19-43: arr0[k] = G[k0, k0, k1, k1, ...] of the vanilla
    tensor on the interleaved triple."""
    from conftest import diagonal_cases

    g = diagonal_golden
    for n in diagonal_cases(g, "amps"):
        A, B, cut = g[f"{n}/A"], g[f"{n}/B"], tuple(int(x) for x in g[f"{n}/cutoffs"])
        if B.ndim > 1 or np.prod(cut) ** 2 > 2e5:
            continue
        G = oracle.vanilla(tuple(x for x in cut for _ in range(2)), A, B, g[f"{n}/G0"])
        diag = np.array([G[tuple(i for k in idx for i in (k, k))] for idx in np.ndindex(*cut)]).reshape(cut)
        arr0 = oracle.diagonal_amps(A, B, g[f"{n}/G0"], cut)[0]
        assert np.allclose(arr0, diag, rtol=1e-10, atol=1e-14), n


def test_diagonal_grad_central_differences(diagonal_golden):
    """dA and dB of the oracle's Jacobians against central differences of its own amplitudes."""
    from conftest import diagonal_cases

    g = diagonal_golden
    n = diagonal_cases(g, "grad")[1]
    A, B, G0, cut = g[f"{n}/A"], g[f"{n}/B"], g[f"{n}/G0"], tuple(g[f"{n}/cutoffs"])
    _, dA, dB = oracle.diagonal_grad(A, B, G0, cut)
    h = 1e-6
    for (p, q) in ((0, 0), (1, 2), (3, 0)):
        E = np.zeros_like(A)
        E[p, q] = h
        fd = (oracle.diagonal_amps(A + E, B, G0, cut)[0] - oracle.diagonal_amps(A - E, B, G0, cut)[0]) / (2 * h)
        assert np.allclose(dA[..., p, q], fd, rtol=1e-6, atol=1e-9)
    for r in (0, 3):
        E = np.zeros_like(B)
        E[r] = h
        fd = (oracle.diagonal_amps(A, B + E, G0, cut)[0] - oracle.diagonal_amps(A, B - E, G0, cut)[0]) / (2 * h)
        assert np.allclose(dB[..., r], fd, rtol=1e-6, atol=1e-9)


def test_fast_diagonal_oracle_matches_reference(diagonal_golden):
    """fast_diagonal (fast_diagonal.py:32-77), vanilla and stable first block, to 1e-14 relative,
    including an output cutoff of 0 where the reference's weight loop ends early (zeros kept)."""
    from conftest import diagonal_cases

    g = diagonal_golden
    try:
        oracle.set_numpy_division(True)
        for n in diagonal_cases(g, "fd"):
            got = oracle.fast_diagonal(g[f"{n}/A"], g[f"{n}/b"], g[f"{n}/c"], int(g[f"{n}/oc"]),
                                       tuple(g[f"{n}/pnr"]), bool(g[f"{n}/stable"]))
            ref = g[f"{n}/out"]
            assert got.shape == ref.shape, n
            assert np.array_equal(got == 0, ref == 0), n
            assert _rel(got, ref) <= 1e-14, (n, _rel(got, ref))
    finally:
        oracle.set_numpy_division(False)


def test_fast_diagonal_equals_vanilla_block(diagonal_golden):
    """tests/test_math/test_fast_diagonal.py:24-45: the leftover-mode blocks equal the vanilla
    tensor's entries G[m, k, n, k] (2 modes) / G[m, k1, k2, n, k1, k2] (3 modes)."""
    from conftest import diagonal_cases

    g = diagonal_golden
    for n in diagonal_cases(g, "fd"):
        pnr, oc = tuple(int(p) for p in g[f"{n}/pnr"]), int(g[f"{n}/oc"])
        L = len(pnr) + 1
        if L > 3 or oc == 0:
            continue
        A, b, c = g[f"{n}/A"], g[f"{n}/b"], g[f"{n}/c"]
        shape = (oc + 1, *(p + 1 for p in pnr))
        G = oracle.vanilla(shape + shape, A, b, c)
        fd = oracle.fast_diagonal(A, b, c, oc, pnr, bool(g[f"{n}/stable"]))
        for q in np.ndindex(*(p + 1 for p in pnr)):
            ref = G[(slice(None), *q, slice(None), *q)]
            assert np.allclose(fd[q], ref, rtol=1e-9, atol=1e-13), (n, q)


def test_leftover_oracle_matches_reference(diagonal_golden):
    """compactFock's leftover-mode strategy (singleLeftoverMode_amps.py, singleLeftoverMode_grad.py):
    the five block arrays and the Jacobians of arr0 against the reference source, to 1e-14 / 1e-13
    relative, with the same elements written."""
    from conftest import diagonal_cases

    g = diagonal_golden
    try:
        oracle.set_numpy_division(True)
        for n in diagonal_cases(g, "lo"):
            A, B, G0, cut = g[f"{n}/A"], g[f"{n}/B"], g[f"{n}/G0"], tuple(g[f"{n}/cutoffs"])
            got = oracle.leftover_amps(A, B, G0, cut)
            for name, x in zip(("arr0", "arr2", "arr1010", "arr1001", "arr1"), got):
                ref = g[f"{n}/{name}"]
                assert x.shape == ref.shape, (n, name)
                assert np.array_equal(x == 0, ref == 0), (n, name)
                assert _rel(x, ref) <= 1e-14, (n, name, _rel(x, ref))
            for name, x in zip(("dG0", "dA", "dB"), oracle.leftover_grad(A, B, G0, cut)):
                ref = g[f"{n}/{name}"]
                assert x.shape == ref.shape, (n, name)
                assert _rel(x, ref) <= 1e-13, (n, name, _rel(x, ref))
    finally:
        oracle.set_numpy_division(False)


def test_leftover_equals_vanilla_blocks(diagonal_golden):
    """tests/test_math/test_compactFock.py:46-69: arr0[m, n, k1, k2, ...] = G[m, n, k1, k1, k2, k2, ...]
    of the vanilla tensor on the interleaved triple."""
    from conftest import diagonal_cases

    g = diagonal_golden
    for n in diagonal_cases(g, "lo"):
        A, B, G0, cut = g[f"{n}/A"], g[f"{n}/B"], g[f"{n}/G0"], tuple(int(x) for x in g[f"{n}/cutoffs"])
        shape = tuple(x for x in cut for _ in range(2))
        if np.prod(shape) > 3e5:
            continue
        G = oracle.vanilla(shape, A, B, G0)
        arr0 = oracle.leftover_amps(A, B, G0, cut)[0]
        for m in range(cut[0]):
            for nn in range(cut[0]):
                for tail in np.ndindex(*cut[1:]):
                    ref = G[(m, nn) + tuple(x for k in tail for x in (k, k))]
                    assert abs(arr0[(m, nn) + tail] - ref) <= 1e-10 * max(1.0, abs(ref)), (n, m, nn, tail)
