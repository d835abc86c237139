"""Generate the golden fixtures of the binomial strategy from the reference's own source.

Runs only where the MrMustard source tree is available (the tests do not run it).  It loads
``mrmustard/math/lattice/strategies/binomial.py`` and the modules it uses (``paths.py``,
``steps.py``, ``pivots.py``, ``neighbors.py``) *unmodified*, by path, under a no-op ``numba``
module (``njit`` is the identity, ``prange`` is ``range``, typed containers are Python
containers, ``tuple_setitem`` rebuilds the tuple), and records
``binomial(local_cutoffs, A, b, c, max_l2, global_cutoff) -> (G, norm)``:

* ``vs_vanilla``: the reference's tests/test_math/test_lattice/test_lattice_functions.py:122-138
  setting (a random 2-mode ket, local cutoffs (5, 5), max_l2 0.9999, global cutoff 12);
* ``ket*``: normalised random kets, M = 1..4, with early stops at several max_l2 values
  (0.5 ... 0.99999) and global cutoffs below and above the local ones;
* ``full*``: max_l2 above 1 (no early stop), so only the global cutoff limits the fill.

Usage (from the repository root)::

    python tests/golden/make_binomial_golden.py /path/to/mrmustard-source
"""

from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np

sys.dont_write_bytecode = True  # the reference tree must stay untouched
HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent.parent))

from make_golden import _install_shims  # noqa: E402


def _install_numba_extras():
    numba = sys.modules["numba"]

    class TypedList(list):
        @staticmethod
        def empty_list(*args, **kwargs):
            return TypedList()

    class TypedDict(dict):
        @staticmethod
        def empty(*args, **kwargs):
            return TypedDict()

    typed = types.ModuleType("numba.typed")
    typed.List = TypedList
    typed.Dict = TypedDict
    ntypes = types.ModuleType("numba.types")
    for name in ("int64", "complex128", "float64"):
        setattr(ntypes, name, object())
    ntypes.UniTuple = lambda *a, **k: object()
    ntypes.ListType = lambda *a, **k: object()
    ntypes.DictType = lambda *a, **k: object()
    numba.typed = typed
    numba.types = ntypes
    numba.typeof = lambda x: object()
    sys.modules["numba.typed"] = typed
    sys.modules["numba.types"] = ntypes
    unsafe_tuple = types.ModuleType("numba.cpython.unsafe.tuple")
    unsafe_tuple.tuple_setitem = lambda t, i, v: t[:i] + (v,) + t[i + 1:]
    for name in ("numba.cpython", "numba.cpython.unsafe"):
        mod = types.ModuleType(name)
        mod.__path__ = []
        sys.modules[name] = mod
    sys.modules["numba.cpython.unsafe.tuple"] = unsafe_tuple


def load_binomial(ref_root: Path):
    _install_shims()
    _install_numba_extras()
    lattice = ref_root / "mrmustard" / "math" / "lattice"
    for name, path in (("mrmustard.math", [str(lattice.parent)]), ("mrmustard.math.lattice", [str(lattice)]),
                       ("mrmustard.math.lattice.strategies", [str(lattice / "strategies")])):
        mod = types.ModuleType(name)
        mod.__path__ = path
        sys.modules[name] = mod
    import importlib

    return importlib.import_module("mrmustard.math.lattice.strategies.binomial")


def main(ref_root: str):
    ref = load_binomial(Path(ref_root))
    import oracle

    out, names = {}, []

    def case(name, cutoffs, A, b, c, max_l2, global_cutoff):
        cutoffs = tuple(int(x) for x in cutoffs)
        G, norm = ref.binomial(cutoffs, np.asarray(A, np.complex128), np.asarray(b, np.complex128),
                               np.complex128(c), max_l2, global_cutoff)
        out[f"{name}/A"], out[f"{name}/b"], out[f"{name}/c"] = np.asarray(A, np.complex128), np.asarray(b, np.complex128), np.complex128(c)
        out[f"{name}/shape"] = np.array(cutoffs, np.int64)
        out[f"{name}/params"] = np.array([max_l2, global_cutoff], np.float64)
        out[f"{name}/G"] = G
        out[f"{name}/norm"] = np.float64(norm)
        names.append(name)

    def ket(M, seed, smax=0.6, sigma=0.6):
        from scipy.stats import unitary_group

        rng = np.random.default_rng(seed)
        U = unitary_group.rvs(M, random_state=seed) if M > 1 else np.exp(1j * rng.uniform(0, 6, (1, 1)))
        A = (U * rng.uniform(0.0, smax, M)) @ U.T
        b = sigma * (rng.standard_normal(M) + 1j * rng.standard_normal(M)) / np.sqrt(2)
        cut = {1: 150, 2: 80, 3: 40, 4: 24, 5: 14, 6: 9, 8: 5}[M]
        G = oracle.vanilla((cut,) * M, A, b, 1.0 + 0j)
        return A, b, 1.0 / np.sqrt(np.sum(np.abs(G) ** 2))

    A, b, c = ket(2, 42)
    case("vs_vanilla", (5, 5), A, b, c, 0.9999, 12)
    for M, cut in ((1, (30,)), (2, (12, 9)), (3, (7, 8, 6)), (4, (5, 4, 6, 3))):
        A, b, c = ket(M, 100 + M)
        for k, (l2, gc) in enumerate(((0.5, 100), (0.9, 100), (0.99999, 100), (0.999, sum(cut) // 2),
                                      (0.99, sum(cut) - M + 1))):
            case(f"ket{M}_{k}", cut, A, b, c, l2, gc)
        case(f"full{M}", cut, A, b, c, 2.0, sum(cut) - M + 1)

    def save(fname):
        out["names"] = np.array(names)
        np.savez(HERE / fname, **out)
        for n in names:
            G = out[f"{n}/G"]
            filled = int(np.count_nonzero(G))
            print(n, tuple(out[f"{n}/shape"]), "norm", float(out[f"{n}/norm"]), "filled", filled, "of", G.size)

    save("binomial_golden.npz")

    # D = 5, 6, 8 in a second file read only by the oracle's tests (the GPU is checked against the
    # oracle there).  (`case` writes into whatever `out` and `names` are bound to.)
    out, names = {}, []
    for M, cut in ((5, (3, 2, 3, 2, 3)), (6, (2, 3, 2, 2, 3, 2)), (8, (2, 2, 2, 2, 2, 2, 2, 2))):
        A, b, c = ket(M, 100 + M)
        gc = sum(cut) - M + 1
        case(f"full{M}", cut, A, b, c, 2.0, gc)
        full = float(out[f"full{M}/norm"])  # the small cutoffs hold only part of the state's norm
        for k, (l2, g) in enumerate(((0.3 * full, gc), (0.7 * full, gc), (0.95 * full, gc), (2.0, sum(cut) // 2))):
            case(f"ket{M}_{k}", cut, A, b, c, l2, g)
    save("binomial_golden_many.npz")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
