"""Generate the golden fixtures of the diagonal strategies from the reference's own source.

Runs only where the MrMustard source tree is available (the tests do not run it).  It loads
``mrmustard/math/lattice/strategies/compactFock/{inputValidation,diagonal_amps,diagonal_grad,
singleLeftoverMode_amps,singleLeftoverMode_grad,helperFunctions}.py`` and
``strategies/fast_diagonal.py`` (with ``vanilla/``) *unmodified*, by path, under the no-op
``numba`` module of ``make_golden.py`` / ``make_binomial_golden.py``, and records:

* ``amps*``: ``hermite_multidimensional_diagonal(A, B, G0, cutoffs)`` -> (arr0, arr2, arr1010,
  arr1001, arr1) for M = 1..4, with and without a batch axis on B;
* ``grad*``: ``grad_hermite_multidimensional_diagonal(A, B, G0, *amps)`` -> (dG0, dA, dB);
* ``lo*``: ``hermite_multidimensional_1leftoverMode(A, B, G0, cutoffs)`` -> (arr0, arr2, arr1010,
  arr1001, arr1) and ``grad_hermite_multidimensional_1leftoverMode`` -> (dG0, dA, dB), M = 2..4
  (cutoffs[0] is the leftover mode's);
* ``fd*``: ``fast_diagonal(A, b, c, output_cutoff, pnr_cutoffs, stable)``, L = 2..4, both
  variants, including the reference tests' shapes (tests/test_math/test_fast_diagonal.py:24-45)
  and an output cutoff of 0, where the reference's weight loop (fast_diagonal.py:70) stops
  before the highest weights.

A is a complex symmetric matrix of spectral norm < 0.9 built from a density-matrix triple
(conj(-A) of a mixed Gaussian state, as tests/test_math/test_compactFock.py:19-43 passes it).

Usage (from the repository root)::

    python tests/golden/make_diagonal_golden.py /path/to/mrmustard-source
"""

from __future__ import annotations

import importlib
import sys
import types
from pathlib import Path

import numpy as np

sys.dont_write_bytecode = True  # the reference tree must stay untouched
HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent.parent))

from make_binomial_golden import _install_numba_extras  # noqa: E402
from make_golden import _install_shims  # noqa: E402


def load(ref_root: Path):
    _install_shims()
    _install_numba_extras()
    sys.modules["numba"].int64 = object()
    lattice = ref_root / "mrmustard" / "math" / "lattice"
    strat = lattice / "strategies"
    for name, path in (("mrmustard.math", [str(lattice.parent)]), ("mrmustard.math.lattice", [str(lattice)]),
                       ("mrmustard.math.lattice.strategies", [str(strat)]),
                       ("mrmustard.math.lattice.strategies.compactFock", [str(strat / "compactFock")])):
        mod = types.ModuleType(name)
        mod.__path__ = path
        sys.modules[name] = mod
    iv = importlib.import_module("mrmustard.math.lattice.strategies.compactFock.inputValidation")
    van = importlib.import_module("mrmustard.math.lattice.strategies.vanilla")
    sys.modules["mrmustard.math.lattice.strategies"].vanilla_numba = van.vanilla_numba
    sys.modules["mrmustard.math.lattice.strategies"].stable_numba = van.stable_numba
    fd = importlib.import_module("mrmustard.math.lattice.strategies.fast_diagonal")
    return iv, fd


def dm_triple(M, seed, r_max=0.6, t_max=0.3, beta=0.4):
    """(A, b, c) of a mixed Gaussian state in Bargmann order (all bra modes, then all ket modes),
    with A = [[conj(K), C^T], [C, K]]: K = U diag(tanh r) U^T (squeezing), C = V diag(t) V^dagger
    (thermal part), b displacement-like.  Returns conj(-A), conj(b), conj(c) as the tests pass it."""
    from scipy.stats import unitary_group

    rng = np.random.default_rng(seed)
    U = unitary_group.rvs(M, random_state=rng) if M > 1 else np.exp(1j * rng.uniform(0, 6, (1, 1)))
    V = unitary_group.rvs(M, random_state=rng) if M > 1 else np.ones((1, 1))
    K = (U * np.tanh(rng.uniform(0.05, r_max, M))) @ U.T
    Cm = (V * rng.uniform(0.0, t_max, M)) @ V.conj().T
    A = np.block([[K.conj(), Cm.T], [Cm, K]])
    bk = beta * (rng.standard_normal(M) + 1j * rng.standard_normal(M))
    b = np.concatenate([bk.conj(), bk])
    c = np.exp(-0.5 * np.sum(np.abs(bk) ** 2)) * np.prod(np.cosh(rng.uniform(0.05, r_max, M))) ** -0.5
    return np.conj(-A).astype(np.complex128), np.conj(b).astype(np.complex128), np.complex128(np.conj(c))


def interleave(A, b):
    """reorder_AB_bargmann (backend_numpy.py:367-375): (m0..m_{M-1}, m0'..) -> (m0, m0', m1, m1', ...)."""
    n = A.shape[0]
    o = np.arange(n).reshape(2, -1).T.flatten()
    return A[o][:, o], b[o]


def main(ref_root: str):
    iv, fd = load(Path(ref_root))
    out, names = {}, []

    def put(name, kind, **arrays):
        for k, v in arrays.items():
            out[f"{name}/{k}"] = np.asarray(v)
        out[f"{name}/kind"] = np.array(kind)
        names.append(name)

    for M, cut, batch in ((1, (12,), 0), (2, (6, 5), 0), (3, (4, 5, 3), 0), (4, (3, 3, 4, 2), 0), (2, (5, 4), 3),
                          (3, (3, 3, 3), 2), (1, (1,), 0), (2, (1, 4), 0), (3, (2, 1, 3), 0)):
        A, b, c = dm_triple(M, 100 + 10 * M + len(names))
        Ai, bi = interleave(A, b)
        B = bi if not batch else bi[:, None] * np.linspace(0.5, 1.5, batch)[None, :]
        r = iv.hermite_multidimensional_diagonal(Ai, B, c, cut)
        put(f"amps{len(names)}", "amps", A=Ai, B=B, G0=c, cutoffs=np.array(cut), arr0=r[0], arr2=r[1],
            arr1010=r[2], arr1001=r[3], arr1=r[4])
        if not batch:
            g = iv.grad_hermite_multidimensional_diagonal(Ai, B, c, *r)
            put(f"grad{len(names)}", "grad", A=Ai, B=B, G0=c, cutoffs=np.array(cut), dG0=g[0], dA=g[1], dB=g[2])

    for M, cut in ((2, (5, 6)), (3, (4, 3, 4)), (4, (3, 2, 3, 2)), (2, (1, 4)), (3, (4, 1, 3)), (2, (6, 1))):
        A, b, c = dm_triple(M, 200 + 10 * M + len(names))
        Ai, bi = interleave(A, b)
        r = iv.hermite_multidimensional_1leftoverMode(Ai, bi, c, cut)
        g = iv.grad_hermite_multidimensional_1leftoverMode(Ai, bi, c, *r)
        put(f"lo{len(names)}", "lo", A=Ai, B=bi, G0=c, cutoffs=np.array(cut), arr0=r[0], arr2=r[1], arr1010=r[2],
            arr1001=r[3], arr1=r[4], dG0=g[0], dA=g[1], dB=g[2])

    for L, oc, pnr, seed in ((2, 5, (10,), 1), (3, 3, (4, 5), 2), (2, 8, (3,), 3), (3, 4, (2, 2), 4),
                             (4, 2, (2, 1, 2), 5), (3, 0, (2, 2), 6), (2, 0, (3,), 7), (4, 1, (1, 1, 1), 8)):
        A, b, c = dm_triple(L, 500 + seed)
        for stable in (False, True):
            G = fd.fast_diagonal(A, b, c, oc, pnr, stable=stable)
            put(f"fd{len(names)}", "fd", A=A, b=b, c=c, oc=np.int64(oc), pnr=np.array(pnr), stable=np.int64(stable),
                out=G)

    out["names"] = np.array(names)
    np.savez_compressed(HERE / "diagonal_golden.npz", **out)
    for n in names:
        print(n, str(out[f"{n}/kind"]))

    # M = 5, 6 in a second file read only by the oracle's tests (the GPU is checked against the
    # oracle there).  (`put` writes into whatever `out` and `names` are bound to.)
    out, names = {}, []
    for M, cut in ((5, (3, 2, 2, 3, 2)), (6, (2, 2, 2, 2, 2, 2))):
        A, b, c = dm_triple(M, 700 + M)
        Ai, bi = interleave(A, b)
        r = iv.hermite_multidimensional_diagonal(Ai, bi, c, cut)
        put(f"amps{len(names)}", "amps", A=Ai, B=bi, G0=c, cutoffs=np.array(cut), arr0=r[0], arr2=r[1],
            arr1010=r[2], arr1001=r[3], arr1=r[4])
        g = iv.grad_hermite_multidimensional_diagonal(Ai, bi, c, *r)
        put(f"grad{len(names)}", "grad", A=Ai, B=bi, G0=c, cutoffs=np.array(cut), dG0=g[0], dA=g[1], dB=g[2])
    for M, cut in ((5, (3, 2, 2, 2, 2)),):
        A, b, c = dm_triple(M, 800 + M)
        Ai, bi = interleave(A, b)
        r = iv.hermite_multidimensional_1leftoverMode(Ai, bi, c, cut)
        g = iv.grad_hermite_multidimensional_1leftoverMode(Ai, bi, c, *r)
        put(f"lo{len(names)}", "lo", A=Ai, B=bi, G0=c, cutoffs=np.array(cut), arr0=r[0], arr2=r[1], arr1010=r[2],
            arr1001=r[3], arr1=r[4], dG0=g[0], dA=g[1], dB=g[2])
    for L, oc, pnr, seed in ((5, 2, (2, 1, 2, 1), 21), (6, 1, (1, 1, 1, 1, 1), 22)):
        A, b, c = dm_triple(L, 900 + seed)
        for stable in (False, True):
            G = fd.fast_diagonal(A, b, c, oc, pnr, stable=stable)
            put(f"fd{len(names)}", "fd", A=A, b=b, c=c, oc=np.int64(oc), pnr=np.array(pnr), stable=np.int64(stable),
                out=G)
    out["names"] = np.array(names)
    np.savez_compressed(HERE / "diagonal_golden_many.npz", **out)
    for n in names:
        print(n, str(out[f"{n}/kind"]))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
