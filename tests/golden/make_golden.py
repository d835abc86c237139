"""Generate the golden fixtures of the Hermite hot path from the reference's own source.

This script runs only where the MrMustard source tree is available (it is not
needed, and not run, by the tests).  It loads the reference's
``mrmustard/math/lattice/strategies/vanilla/{core,batch,gradients}.py`` and
``strategies/displacement.py`` *unmodified*, by path, under a no-op ``numba``
module (``njit`` is the identity, ``prange`` is ``range``), so the exact
reference algorithm runs as CPython + numpy.  Every case writes its inputs and
the reference outputs into ``tests/golden/hermite_golden.npz``.

Cases (each cites the reference test it mirrors):

* ``kat1d``: 1-D renormalised Hermite polynomials, A = -2, b = 2x
  (tests/test_math/test_special.py:23-36).
* ``rt2``/``rt3``: ``random_triple(n, seed=673)``, shape 4^n, vanilla + stable + VJP
  (tests/test_math/test_lattice/test_vanilla.py:24-87).
* ``batch``: ``random_triple(3, (2,), seed=673)``, shape (1,2,3), batched forward and VJP
  (test_vanilla.py:89-162).
* ``cfg1``: 3-mode pure Gaussian state (Takagi form A = Q diag(s) Q^T), shape 20^3.
* ``ragged*``: uneven shapes with unit axes, D = 1..4.
* ``dm4``: 4-index density-matrix style triple (complex symmetric A, spectral norm 0.89), shape 6^4.
* ``dgate``: displacement gate alpha = 4+4j at 60x60, vanilla + stable + the reference's
  closed-form ``displacement`` strategy (tests/test_math/test_lattice/test_lattice_functions.py:141-152).
* ``many5``..``many8`` (in ``hermite_golden_many.npz``): ``random_triple(D)`` at D = 5..8 with small
  uneven shapes, vanilla + stable + VJP.

Usage (from the repository root)::

    python tests/golden/make_golden.py /path/to/mrmustard-source
"""

from __future__ import annotations

import importlib.util
import sys
import types
from pathlib import Path

import numpy as np

sys.dont_write_bytecode = True  # the reference tree must stay untouched

HERE = Path(__file__).resolve().parent


def _install_shims():
    numba = types.ModuleType("numba")

    def njit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    numba.njit = njit
    numba.prange = range
    numba.jit = njit
    sys.modules["numba"] = numba
    mm = types.ModuleType("mrmustard")
    mm.__path__ = []
    utils = types.ModuleType("mrmustard.utils")
    utils.__path__ = []
    typing = types.ModuleType("mrmustard.utils.typing")
    for name in ("ComplexTensor", "ComplexMatrix", "ComplexVector", "RealVector"):
        setattr(typing, name, np.ndarray)
    sys.modules.setdefault("mrmustard", mm)
    sys.modules["mrmustard.utils"] = utils
    sys.modules["mrmustard.utils.typing"] = typing


def load_reference(ref_root: Path):
    """Load the reference's vanilla strategy package and displacement module by path."""
    _install_shims()
    strat = ref_root / "mrmustard" / "math" / "lattice" / "strategies"
    pkg_name = "_ref_vanilla"
    pkg = types.ModuleType(pkg_name)
    pkg.__path__ = [str(strat / "vanilla")]
    sys.modules[pkg_name] = pkg
    mods = {}
    for name in ("core", "batch", "gradients"):
        spec = importlib.util.spec_from_file_location(f"{pkg_name}.{name}", strat / "vanilla" / f"{name}.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[spec.name] = mod
        spec.loader.exec_module(mod)
        mods[name] = mod
    spec = importlib.util.spec_from_file_location("_ref_displacement", strat / "displacement.py")
    disp = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(disp)
    mods["displacement"] = disp
    return mods


class _WrapArray(np.ndarray):
    """ndarray whose flat reads below ``-len`` return 0.

    ``vanilla_vjp_numba`` (gradients.py:64-76) reads ``G_lin[pivot - strides[j]]`` with indices
    that can fall below ``-len`` for shapes with short axes; numba (no bounds checking) reads
    whatever lies there and multiplies it by ``SQRT[0] = 0``.  CPython raises instead, so the
    fixture generator returns 0 for those reads, which is the value numba's product takes.
    """

    def __getitem__(self, idx):
        if isinstance(idx, (int, np.integer)) and self.ndim == 1 and idx < -self.shape[0]:
            return np.complex128(0.0)
        return super().__getitem__(idx)


def _wrap(G):
    return np.ascontiguousarray(G).view(_WrapArray)


def random_triple(n, batch=(), seed=None):
    """Same construction as tests/test_math/test_lattice/test_vanilla.py:24-35."""
    rng = np.random.RandomState(seed) if seed is not None else np.random
    A = rng.random((*batch, n, n)) + 1j * rng.random((*batch, n, n))
    A = A + np.swapaxes(A, -1, -2)
    A /= np.abs(np.linalg.eigvals(A)).max() + 0.2
    b = rng.random((*batch, n)) + 1j * rng.random((*batch, n))
    c = rng.random(batch) + 1j * rng.random(batch)
    return A, b, c


def takagi_triple(D, smax, seed, sigma=0.3):
    """Pure-state Bargmann triple: A = Q diag(s) Q^T (Q Haar unitary), b complex normal."""
    from scipy.stats import unitary_group

    rng = np.random.default_rng(seed)
    Q = unitary_group.rvs(D, random_state=seed) if D > 1 else np.exp(1j * rng.uniform(0, 2 * np.pi, (1, 1)))
    s = rng.uniform(0.0, smax, D)
    A = (Q * s) @ Q.T
    b = sigma * (rng.standard_normal(D) + 1j * rng.standard_normal(D)) / np.sqrt(2)
    return A.astype(np.complex128), b.astype(np.complex128), np.complex128(1.0)


def dm_triple(D, norm, seed, sigma=0.3):
    """Complex symmetric A scaled to a given spectral norm (density-matrix style)."""
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((D, D)) + 1j * rng.standard_normal((D, D))
    A = X + X.T
    A *= norm / np.linalg.norm(A, 2)
    b = sigma * (rng.standard_normal(D) + 1j * rng.standard_normal(D)) / np.sqrt(2)
    return A.astype(np.complex128), b.astype(np.complex128), np.complex128(1.0)


def cnormal(shape, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex128)


def main(ref_root: str):
    ref = load_reference(Path(ref_root))
    core, batch, grads, disp = ref["core"], ref["batch"], ref["gradients"], ref["displacement"]
    out = {}

    def single(name, A, b, c, shape, with_stable=True, with_vjp=True, seed=0):
        shape = tuple(int(s) for s in shape)
        out[f"{name}/A"] = np.asarray(A, np.complex128)
        out[f"{name}/b"] = np.asarray(b, np.complex128)
        out[f"{name}/c"] = np.complex128(c)
        out[f"{name}/shape"] = np.array(shape, np.int64)
        G = core.vanilla_numba(shape, np.asarray(A), np.asarray(b), np.complex128(c))
        out[f"{name}/G"] = G
        if with_stable:
            out[f"{name}/G_stable"] = core.stable_numba(shape, np.asarray(A), np.asarray(b), np.complex128(c))
        if with_vjp:
            g = cnormal(shape, 1000 + seed)
            dA, db, dc = grads.vanilla_vjp_numba(_wrap(G), np.complex128(c), g)
            out[f"{name}/dLdG"] = g
            out[f"{name}/dA"] = dA
            out[f"{name}/db"] = db
            out[f"{name}/dc"] = np.complex128(dc)

    # 1-D known-answer test: renormalised physicists' Hermite polynomials.
    xs = np.arange(-1, 1, 0.1)
    kat = np.array([core.vanilla_numba((5,), -2 * np.ones((1, 1), complex), 2 * np.array([x0], complex), 1 + 0j) for x0 in xs])
    out["kat1d/x"] = xs
    out["kat1d/G"] = kat

    A, b, c = random_triple(2, (), seed=673)
    single("rt2", A, b, c, (4, 4), seed=2)
    A, b, c = random_triple(3, (), seed=673)
    single("rt3", A, b, c, (4, 4, 4), seed=3)

    A, b, c = random_triple(3, (2,), seed=673)
    shape = (1, 2, 3)
    Gb = batch.vanilla_batch_numba(shape, A, b, c)
    Gbs = batch.vanilla_batch_numba(shape, A, b, c, True)
    g = cnormal(Gb.shape, 1234)
    dA, db, dc = grads.vanilla_batch_vjp_numba(_wrap(Gb), c, g)
    out.update({"batch/A": A, "batch/b": b, "batch/c": c, "batch/shape": np.array(shape, np.int64),
                "batch/G": Gb, "batch/G_stable": Gbs, "batch/dLdG": g, "batch/dA": dA, "batch/db": db, "batch/dc": dc})

    A, b, c = takagi_triple(3, 0.8, seed=20251)
    single("cfg1", A, b, c, (20, 20, 20), seed=1)

    for k, (D, shape, seed) in enumerate([(1, (6,), 11), (2, (1, 7), 12), (2, (7, 1), 13), (3, (5, 1, 4), 14),
                                          (4, (3, 1, 4, 2), 15), (4, (2, 3, 2, 5), 16), (3, (1, 1, 1), 17)]):
        A, b, c = random_triple(D, (), seed=seed)
        single(f"ragged{k}", A, b, c, shape, seed=10 + k)

    A, b, c = dm_triple(4, 0.89, seed=404)
    single("dm4", A, b, c, (6, 6, 6, 6), seed=4)

    alpha = 4.0 + 4.0j
    A = np.array([[0, 1], [1, 0]], np.complex128)
    b = np.array([alpha, -np.conj(alpha)], np.complex128)
    c = np.complex128(np.exp(-abs(alpha) ** 2 / 2))
    single("dgate", A, b, c, (60, 60), with_vjp=False)
    out["dgate/displacement"] = disp.displacement((60, 60), alpha)

    np.savez_compressed(HERE / "hermite_golden.npz", **out)
    print("wrote", HERE / "hermite_golden.npz", "with", len(out), "arrays")

    # D = 5..8 (the GPU library's largest mode counts), small uneven shapes, in a second file read
    # only by the oracle's tests: the GPU is checked against the oracle at these D.  (`single`
    # writes into whatever `out` is bound to.)
    out = {}
    for D, shape, seed in ((5, (3, 2, 3, 1, 2), 51), (6, (2, 2, 3, 2, 1, 2), 52), (7, (2, 1, 2, 2, 2, 1, 2), 53),
                           (8, (2, 2, 1, 2, 2, 1, 2, 2), 54)):
        A, b, c = random_triple(D, (), seed=seed)
        single(f"many{D}", A, b, c, shape, seed=50 + D)
    np.savez_compressed(HERE / "hermite_golden_many.npz", **out)
    print("wrote", HERE / "hermite_golden_many.npz", "with", len(out), "arrays")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
