"""Generate the golden fixtures of autoshape from the reference's own source.

Runs only where the MrMustard source tree is available (the tests do not run it).
It loads ``mrmustard/math/lattice/autoshape.py`` *unmodified*, by path, under the
same no-op ``numba`` module as ``make_golden.py``, and records the reference's
``autoshape_numba(A, b, c, max_prob, max_shape, min_shape)`` on density-matrix
triples (2M x 2M A, 2M b, scalar c; first M variables the bra copy, last M the
ket copy, as ``State.auto_shape`` builds them with ``ansatz.conj & ansatz``,
lab/states/base.py:383-430).

Cases:

* ``coh1``: Coherent(alpha=1) -> (8,), the reference's tests/test_lab/test_states/test_ket.py:98-100
  and test_dm.py:82-84; ``vac``: the vacuum -> (1,), test_coherent.py:74-75 (both asserted here too).
* ``sq*``: squeezed vacua rotated by a Haar-random passive unitary, M = 1..4 (normalised in closed form).
* ``coh*``: coherent product states rotated by a passive unitary (A = 0: the reduction inverts -X).
* ``gauss*``: pure Gaussian states with A and b both non-zero, normalised with the oracle's Fock sums.
* ``thermal*``: mixed states with a Hermitian bra-ket block.
* ``clip*``, ``prob*``: the max_shape / min_shape clips and other max_prob thresholds.
* ``rand*``: random pure states (M = 1..5) and pure states with an added bra-ket block.
* ``sq6``..``sq8``, ``coh6``..``coh8`` (in ``autoshape_golden_many.npz``): M = 6..8.

Usage (from the repository root)::

    python tests/golden/make_autoshape_golden.py /path/to/mrmustard-source
"""

from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np

sys.dont_write_bytecode = True  # the reference tree must stay untouched
HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent.parent))

from make_golden import _install_shims  # noqa: E402


def load_autoshape(ref_root: Path):
    _install_shims()
    path = ref_root / "mrmustard" / "math" / "lattice" / "autoshape.py"
    spec = importlib.util.spec_from_file_location("_ref_autoshape", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def haar(M, seed):
    from scipy.stats import unitary_group

    return unitary_group.rvs(M, random_state=seed) if M > 1 else np.exp(1j * np.array([[0.3 + seed]]))


def ket_to_dm(A, b, c):
    """(A, b, c) of a ket -> the density-matrix triple conj & ket (block-diagonal A)."""
    M = len(b)
    Adm = np.zeros((2 * M, 2 * M), np.complex128)
    Adm[:M, :M] = np.conj(A)
    Adm[M:, M:] = A
    return Adm, np.concatenate([np.conj(b), b]).astype(np.complex128), np.complex128(abs(c) ** 2)


def fock_norm2(A, b, c, cutoff):
    """sum |G|^2 of the ket's Fock amplitudes up to `cutoff` per mode (C oracle)."""
    import oracle

    G = oracle.vanilla((cutoff,) * len(b), A, b, c)
    return float(np.sum(np.abs(G) ** 2))


def main(ref_root: str):
    ref = load_autoshape(Path(ref_root))
    out = {}
    names = []

    def case(name, A, b, c, max_prob=0.99999, max_shape=50, min_shape=1):
        A = np.ascontiguousarray(A, np.complex128)
        b = np.ascontiguousarray(b, np.complex128)
        shape = ref.autoshape_numba(A, b, np.complex128(c), max_prob, max_shape, min_shape)
        out[f"{name}/A"], out[f"{name}/b"], out[f"{name}/c"] = A, b, np.complex128(c)
        out[f"{name}/params"] = np.array([max_prob, max_shape, min_shape], np.float64)
        out[f"{name}/shape"] = np.asarray(shape, np.int64)
        names.append(name)
        return tuple(int(s) for s in shape)

    # known answers from the reference's own tests
    a = 1.0
    assert case("coh1", *ket_to_dm(np.zeros((1, 1)), np.array([a]), np.exp(-abs(a) ** 2 / 2))) == (8,)
    assert case("vac", *ket_to_dm(np.zeros((1, 1)), np.zeros(1), 1.0)) == (1,)

    # squeezed vacua rotated by a passive unitary: A = U diag(-e^{i phi} tanh r) U^T, c = prod cosh(r)^-1/2
    for M in (1, 2, 3, 4):
        rng = np.random.default_rng(100 + M)
        r = rng.uniform(0.1, 0.8, M)
        phi = rng.uniform(0, 2 * np.pi, M)
        U = haar(M, 200 + M)
        A = U @ np.diag(-np.exp(1j * phi) * np.tanh(r)) @ U.T
        case(f"sq{M}", *ket_to_dm(A, np.zeros(M), np.prod(np.cosh(r) ** -0.5)))

    # coherent products rotated by a passive unitary (A = 0)
    for M in (2, 3, 4):
        rng = np.random.default_rng(300 + M)
        alpha = rng.normal(0, 1.0, M) + 1j * rng.normal(0, 1.0, M)
        U = haar(M, 400 + M)
        case(f"coh{M}", *ket_to_dm(np.zeros((M, M)), U @ alpha, np.exp(-np.sum(np.abs(alpha) ** 2) / 2)))

    # pure Gaussian states with A and b non-zero, normalised by their Fock sums
    for M, cut in ((1, 120), (2, 70), (3, 40), (4, 26)):
        rng = np.random.default_rng(500 + M)
        U = haar(M, 600 + M)
        A = (U * rng.uniform(0.0, 0.55, M)) @ U.T
        b = 0.6 * (rng.standard_normal(M) + 1j * rng.standard_normal(M)) / np.sqrt(2)
        c = 1.0 / np.sqrt(fock_norm2(A, b, 1.0 + 0j, cut))
        case(f"gauss{M}", *ket_to_dm(A, b, c))

    # mixed (thermal-like) states: bra-ket block C = U diag(t) U^dagger, c = prod(1 - t)
    for M in (1, 2, 3):
        rng = np.random.default_rng(700 + M)
        t = rng.uniform(0.05, 0.6, M)
        U = haar(M, 800 + M)
        Cm = U @ np.diag(t) @ U.conj().T
        Adm = np.zeros((2 * M, 2 * M), np.complex128)
        Adm[:M, M:] = Cm.T
        Adm[M:, :M] = Cm
        case(f"thermal{M}", Adm, np.zeros(2 * M), np.prod(1 - t))

    # clipping and thresholds
    big = 5.0 + 2.0j
    case("clip_max", *ket_to_dm(np.zeros((1, 1)), np.array([big]), np.exp(-abs(big) ** 2 / 2)))
    case("clip_max20", *ket_to_dm(np.zeros((1, 1)), np.array([big]), np.exp(-abs(big) ** 2 / 2)), max_shape=20)
    case("clip_min", *ket_to_dm(np.zeros((1, 1)), np.zeros(1), 1.0), min_shape=3)
    rng = np.random.default_rng(900)
    U = haar(3, 901)
    A = (U * rng.uniform(0.0, 0.5, 3)) @ U.T
    b = 0.5 * (rng.standard_normal(3) + 1j * rng.standard_normal(3))
    c = 1.0 / np.sqrt(fock_norm2(A, b, 1.0 + 0j, 40))
    for k, p in enumerate((0.5, 0.9, 0.999, 0.9999999)):
        case(f"prob{k}", *ket_to_dm(A, b, c), max_prob=p)

    # random states: pure Gaussian (M = 1..5) and mixtures of a pure state with a thermal part
    for k in range(24):
        rng = np.random.default_rng(1000 + k)
        M = 1 + k % 5
        U = haar(M, 1100 + k)
        A = (U * rng.uniform(0.0, 0.6, M)) @ U.T
        b = rng.uniform(0.1, 0.9) * (rng.standard_normal(M) + 1j * rng.standard_normal(M)) / np.sqrt(2)
        cut = {1: 120, 2: 70, 3: 40, 4: 26, 5: 16}[M]
        c = 1.0 / np.sqrt(fock_norm2(A, b, 1.0 + 0j, cut))
        Adm, bdm, cdm = ket_to_dm(A, b, c)
        if k % 3 == 2:  # add a bra-ket block: a mixed state's triple (no longer normalised)
            t = rng.uniform(0.05, 0.3, M)
            Cm = U @ np.diag(t) @ U.conj().T
            Adm[:M, M:] = Cm.T
            Adm[M:, :M] = Cm
        case(f"rand{k}", Adm, bdm, cdm, max_prob=[0.99999, 0.999, 0.99][k % 3], max_shape=[50, 30, 80][k % 3])

    out["names"] = np.array(names)
    np.savez(HERE / "autoshape_golden.npz", **out)
    for n in names:
        print(n, tuple(out[f"{n}/shape"]))

    # M = 6..8 (the GPU library's largest mode counts), in a second file read only by the oracle's
    # tests: squeezed vacua and coherent products rotated by a passive unitary (closed-form norms).
    # (`case` writes into whatever `out` and `names` are bound to.)
    out, names = {}, []
    for M in (6, 7, 8):
        rng = np.random.default_rng(1300 + M)
        r = rng.uniform(0.1, 0.6, M)
        phi = rng.uniform(0, 2 * np.pi, M)
        U = haar(M, 1400 + M)
        A = U @ np.diag(-np.exp(1j * phi) * np.tanh(r)) @ U.T
        case(f"sq{M}", *ket_to_dm(A, np.zeros(M), np.prod(np.cosh(r) ** -0.5)))
        alpha = 0.8 * (rng.normal(0, 1.0, M) + 1j * rng.normal(0, 1.0, M))
        V = haar(M, 1500 + M)
        case(f"coh{M}", *ket_to_dm(np.zeros((M, M)), V @ alpha, np.exp(-np.sum(np.abs(alpha) ** 2) / 2)))
    out["names"] = np.array(names)
    np.savez(HERE / "autoshape_golden_many.npz", **out)
    for n in names:
        print(n, tuple(out[f"{n}/shape"]))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
