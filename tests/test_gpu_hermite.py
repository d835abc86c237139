"""GPU parity of the Hermite hot path: the CUDA library (through its C ABI, via the package's
ctypes layer) against the reference's own outputs (golden fixtures) and the CPU oracle.

Tolerances (max|x - ref| / max|ref| per instance, the metric of the reference's recurrence whose
amplitudes span tens of decades):
  * forward, well-conditioned triples: 1e-13;
  * forward, the 4-index density-matrix triple at cutoff 50 (error grows along the recurrence in
    the reference itself): 1e-12;
  * VJP (sums of up to millions of products, tree-ordered on the GPU, sequential in numba): 1e-12.
"""

from __future__ import annotations

import ctypes

import time

import numpy as np
import pytest
import torch

import mrmustard_gb300 as mm
from conftest import golden_cases
from mrmustard_gb300 import _lib

pytestmark = pytest.mark.gpu

FWD_TOL = 1e-13
FWD_TOL_ILL = 1e-12
VJP_TOL = 1e-12


def rel(x, ref):
    x = x.cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)
    ref = np.asarray(ref)
    den = np.abs(ref).max()
    return float(np.abs(x - ref).max() / den) if den > 0 else float(np.abs(x).max())


def takagi(D, smax, seed, sigma=0.3):
    from scipy.stats import unitary_group

    rng = np.random.default_rng(seed)
    Q = unitary_group.rvs(D, random_state=seed) if D > 1 else np.exp(1j * rng.uniform(0, 2 * np.pi, (1, 1)))
    s = rng.uniform(0, smax, D)
    A = (Q * s) @ Q.T
    b = sigma * (rng.standard_normal(D) + 1j * rng.standard_normal(D)) / np.sqrt(2)
    return A, b, 1.0 + 0j


def dm_triple(D, norm, seed, sigma=0.3):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((D, D)) + 1j * rng.standard_normal((D, D))
    A = X + X.T
    A *= norm / np.linalg.norm(A, 2)
    b = sigma * (rng.standard_normal(D) + 1j * rng.standard_normal(D)) / np.sqrt(2)
    return A, b, 1.0 + 0j


def cn(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


# ---------------------------------------------------------------- golden fixtures
def reference_sensitivity(oracle_lib, fn, shape, A, b, c):
    """How far the reference's own result moves when only its complex/real division is lowered
    differently (numba's true division vs numpy's reciprocal multiply): one ulp per division.
    For ill-conditioned triples this, not 1e-13, is the resolution at which the reference is
    defined."""
    oracle_lib.set_numpy_division(True)
    try:
        x = fn(shape, A, b, c)
    finally:
        oracle_lib.set_numpy_division(False)
    return rel(fn(shape, A, b, c), x)


def test_golden_forward(golden, cuda, oracle_lib):
    for n in golden_cases(golden, ("G", "G_stable")):
        sh = tuple(golden[f"{n}/shape"])
        A, b, c = golden[f"{n}/A"], golden[f"{n}/b"], golden[f"{n}/c"]
        G = mm.vanilla_numba(sh, A, b, c)
        assert G.shape == sh and G.dtype == np.complex128
        if n != "dgate":  # vanilla diverges there in the reference too (|G| ~ 1e7)
            assert rel(G, golden[f"{n}/G"]) < FWD_TOL, n
        tol = FWD_TOL
        if n == "dgate":  # stable Dgate(4+4j): the reference moves by 2.4e-11 under one-ulp changes
            tol = max(FWD_TOL, 10 * reference_sensitivity(oracle_lib, oracle_lib.stable, sh, A, b, c))
        assert rel(mm.stable_numba(sh, A, b, c), golden[f"{n}/G_stable"]) < tol, n


def test_golden_vjp(golden, cuda):
    for n in golden_cases(golden, ("dA",)):
        dA, db, dc = mm.vanilla_vjp_numba(golden[f"{n}/G"], golden[f"{n}/c"], golden[f"{n}/dLdG"])
        assert rel(dA, golden[f"{n}/dA"]) < VJP_TOL, n
        assert rel(db, golden[f"{n}/db"]) < VJP_TOL, n
        assert abs(dc - golden[f"{n}/dc"]) <= VJP_TOL * max(1.0, abs(golden[f"{n}/dc"])), n


def test_golden_batch(golden, cuda):
    sh = tuple(golden["batch/shape"])
    A, b, c = golden["batch/A"], golden["batch/b"], golden["batch/c"]
    assert rel(mm.vanilla_batch_numba(sh, A, b, c), golden["batch/G"]) < FWD_TOL
    assert rel(mm.vanilla_batch_numba(sh, A, b, c, True), golden["batch/G_stable"]) < FWD_TOL
    dA, db, dc = mm.vanilla_batch_vjp_numba(golden["batch/G"], c, golden["batch/dLdG"])
    assert rel(dA, golden["batch/dA"]) < VJP_TOL
    assert rel(db, golden["batch/db"]) < VJP_TOL
    assert rel(dc, golden["batch/dc"]) < VJP_TOL


def test_known_answer_1d(golden, cuda):
    from scipy.special import eval_hermite, factorial

    x = golden["kat1d/x"]
    expected = np.array([eval_hermite(i, x) / np.sqrt(factorial(i)) for i in range(5)]).T
    got = np.array([mm.hermite_renormalized(-2 * np.ones((1, 1)), 2 * np.array([x0]), 1, (5,)) for x0 in x])
    np.testing.assert_allclose(got, expected, atol=1e-12)


def test_conj_views_are_materialised(cuda, oracle_lib):
    """Tensors carrying torch's lazy conjugation bit must reach the kernels conjugated."""
    A, b, c = takagi(2, 0.6, 901)
    shape = (6, 7)
    G = oracle_lib.vanilla(shape, A, b, c)
    g = cn(shape, 902)
    ref = oracle_lib.vjp(G, c, g)
    gt = torch.as_tensor(g.conj(), device=cuda).conj()  # conj view whose values equal g
    assert gt.is_conj()
    got = mm.vanilla_vjp_numba(torch.as_tensor(G, device=cuda), torch.tensor(c, device=cuda), gt)
    assert rel(got[1], ref[1]) < VJP_TOL
    bt = torch.as_tensor(b.conj(), device=cuda).conj()
    Gd = mm.vanilla_numba(shape, torch.as_tensor(A, device=cuda), bt, torch.tensor(c, device=cuda))
    assert rel(Gd, G) < FWD_TOL


def test_stable_dgate_displacement(golden, cuda):
    G = mm.stable_numba((60, 60), golden["dgate/A"], golden["dgate/b"], golden["dgate/c"])
    assert np.allclose(G, golden["dgate/displacement"])


def test_stable_dgate_1000(cuda, oracle_lib):
    """test_lattice_functions.py:141-152 at full size: stable Dgate(4+4j) at 1000x1000."""
    alpha = 4 + 4j
    A = np.array([[0, 1], [1, 0]], complex)
    b = np.array([alpha, -np.conj(alpha)])
    c = np.exp(-abs(alpha) ** 2 / 2)
    with mm.settings(STABLE_FOCK_CONVERSION=True):
        G = mm.hermite_renormalized(A, b, c, (1000, 1000))
    ref = oracle_lib.stable((1000, 1000), A, b, c)
    # the reference itself moves by ~2.7e-9 here under one-ulp changes of its division
    tol = 10 * reference_sensitivity(oracle_lib, oracle_lib.stable, (1000, 1000), A, b, c)
    assert rel(G, ref) < max(tol, 1e-12)
    r, phi = 4.0, 2.0
    A = np.array([[-np.exp(1j * phi) * np.tanh(r), 1 / np.cosh(r)], [1 / np.cosh(r), np.exp(-1j * phi) * np.tanh(r)]])
    with mm.settings(STABLE_FOCK_CONVERSION=True):
        S = mm.hermite_renormalized(A, np.zeros(2), 1 / np.sqrt(np.cosh(r)), (1000, 1000))
    assert np.max(np.abs(S)) < 1


# ---------------------------------------------------------------- configs
def test_cfg1_plain(cuda, oracle_lib):
    A, b, c = takagi(3, 0.8, 101)
    G = mm.vanilla_numba((20, 20, 20), A, b, c)
    ref = oracle_lib.vanilla((20, 20, 20), A, b, c)
    assert G.shape == (20, 20, 20)
    assert rel(G, ref) < FWD_TOL


@pytest.mark.parametrize("case", ["pure40", "dm50"])
def test_cfg2_large_single(cuda, oracle_lib, case):
    if case == "pure40":
        A, b, c = takagi(4, 0.85, 202)
        shape, tol = (40,) * 4, FWD_TOL
    else:
        A, b, c = dm_triple(4, 0.89, 203)
        shape, tol = (50,) * 4, FWD_TOL_ILL
    Gd = mm.device_fwd(torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda),
                       torch.tensor(c, dtype=torch.complex128, device=cuda), shape)
    assert rel(Gd, oracle_lib.vanilla(shape, A, b, c)) < tol


# A single instance of at least 4096 amplitudes whose slab 0 exceeds the 2560-amplitude face region
# runs the dataflow forward (per-range progress words, shared-memory small levels, lane-pair chains);
# those with a smaller slab 0 run the one-cluster kernel (tested below; the forced-schedule test runs
# some of them on the dataflow kernel as well).  Shapes chosen for the corners of its plan:
# a 1-D chain; 2-D; no shared-memory region (an axis longer than 2560); axes of length 1; D = 7, 8;
# a whole tensor's face in shared memory; a level-1 chunk split over more than half the SMs (no
# exclusive SMs); the smallest instances on the grid (4096 .. 8000 amplitudes, the 3-mode cutoff-20
# state among them).
@pytest.mark.parametrize("shape", [(9000,), (300, 40), (4, 5, 3000), (10, 1, 30, 40, 2), (20, 30, 15),
                                   (4, 4, 4, 4, 4, 4, 4), (2, 2, 2, 2, 2, 2, 2, 64), (60, 1, 1, 200),
                                   (3, 10, 10000), (20, 20, 20), (16, 16, 16), (8, 8, 8, 8), (4096,), (64, 70),
                                   (2, 2048), (5, 9, 100)])
def test_single_instance_dataflow_shapes(cuda, oracle_lib, shape):
    A, b, c = takagi(len(shape), 0.8, 900 + sum(shape))
    Gd = mm.device_fwd(torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda),
                       torch.tensor(c, dtype=torch.complex128, device=cuda), shape)
    assert rel(Gd, oracle_lib.vanilla(shape, A, b, c)) < FWD_TOL


# A single instance of at least 1024 amplitudes whose slab 0 (strides[0] amplitudes) fits the
# 2560-amplitude face region runs on one thread-block cluster (slab 0 on CTA 0, level-0 chunks split
# over up to 16 CTAs, distributed shared memory): corners of its plan -- one chunk of level 0
# (shape[0] = 1, 2), the largest slab 0 (2560: 16 CTAs, two amplitudes per lane pair), D = 1, 5, 6, 8,
# a 1-CTA cluster, odd extents.
CLUSTER_SHAPES = [(20, 20, 20), (8, 2560), (1, 40, 40), (2, 30, 30), (3, 4, 5, 6, 7), (1024,), (32, 32),
                  (17, 13, 11), (4, 4, 4, 4, 4, 4), (3, 3, 3, 3, 3, 3, 3, 3), (10, 10, 10, 10), (40, 400)]


@pytest.mark.parametrize("shape", CLUSTER_SHAPES)
def test_single_instance_cluster_shapes(cuda, oracle_lib, shape):
    A, b, _ = takagi(len(shape), 0.8, 1900 + sum(shape))
    c = 0.7 - 0.2j
    Gd = mm.device_fwd(torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda),
                       torch.tensor(c, dtype=torch.complex128, device=cuda), shape)
    assert rel(Gd, oracle_lib.vanilla(shape, A, b, c)) < FWD_TOL


# Large single instances on the dataflow kernel with polled amplitudes (G pre-filled with a pending
# pattern, every input of another CTA polled): the benchmark's 4 x 40 and 4 x 30 states, a cutoff-50
# level 1 (2500 amplitudes per chunk), an extent of 1 on axis 1, D = 3, 5, 6, 7, 8, a 2560-amplitude
# slab.  The halo loads of a chunk go out in batches of at most six: at D = 8 a level-0 amplitude has
# seven possible halo terms (two batches), at 3 x 50^3 four amplitudes per lane pair give twelve.
POLLED_SHAPES = [(6, 40, 40, 40), (30, 30, 30, 30), (3, 50, 50, 50), (5, 3, 1000), (2, 2, 2560),
                (4, 8, 8, 8, 8, 6), (40, 1, 40, 40), (20, 12, 12, 12, 12), (40, 4, 4, 4, 4, 4, 4),
                (12, 4, 4, 4, 4, 4, 4, 4)]


@pytest.mark.parametrize("shape", POLLED_SHAPES)
def test_single_instance_polled_shapes(cuda, oracle_lib, shape):
    A, b, _ = takagi(len(shape), 0.8, 700 + sum(shape))
    c = 0.9 + 0.3j
    Gd = mm.device_fwd(torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda),
                       torch.tensor(c, dtype=torch.complex128, device=cuda), shape)
    assert rel(Gd, oracle_lib.vanilla(shape, A, b, c)) < FWD_TOL


def test_polled_forward_nan_inputs(cuda):
    """NaN inputs carrying the all-ones bit pattern that the polled dataflow forward pre-fills G with
    (in c, which G[0] holds, and in b, which every computed amplitude inherits): the call completes
    (no amplitude is left looking pending, no wait times out) and returns NaNs."""
    pending = np.frombuffer(np.full(8, 0xFF, np.uint8).tobytes(), np.float64)[0]
    shape = (6, 40, 40, 40)
    A, b, _ = takagi(4, 0.8, 811)
    b = b.copy()
    b[1] = complex(pending, pending)
    c = complex(pending, pending)
    t0 = time.perf_counter()
    G = mm.device_fwd(torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda),
                      torch.tensor(c, dtype=torch.complex128, device=cuda), shape)
    torch.cuda.synchronize()
    assert time.perf_counter() - t0 < 1.0
    assert torch.isnan(G.real).all() and torch.isnan(G.imag).all()


_FORCED = """
import sys, numpy as np, torch
sys.path.insert(0, {root!r})
import mrmustard_gb300 as mm
from test_gpu_hermite import takagi
out = {{}}
for shape in {shapes!r}:
    A, b, c = takagi(len(shape), 0.8, 1900 + sum(shape))
    G = mm.device_fwd(torch.as_tensor(A, device='cuda'), torch.as_tensor(b, device='cuda'),
                      torch.tensor(0.7 - 0.2j, dtype=torch.complex128, device='cuda'), shape)
    out['x'.join(map(str, shape))] = G.cpu().numpy()
np.savez({path!r}, **out)
"""


@pytest.mark.parametrize("env", [{"MM_CLUSTER_FWD": "0"}, {"MM_CLUSTER_CTAS": "1"}, {"MM_CLUSTER_CTAS": "3"},
                                 {"MM_CLUSTER_CTAS": "16"}, {"MM_FLOW_POLL": "0"}])
def test_single_instance_forced_schedules(cuda, oracle_lib, tmp_path, env):
    """The same instances with the cluster kernel off (grid-wide dataflow kernel instead), with
    fixed cluster sizes and with the large-instance dataflow on progress words instead of polled
    amplitudes (schedule knobs are read once per process, so each runs in a child)."""
    import os
    import subprocess
    import sys
    from pathlib import Path

    shapes = [(20, 20, 20), (8, 2560), (2, 30, 30), (1024,), (40, 400), (6, 40, 40, 40), (5, 3, 1000)]
    root = str(Path(__file__).resolve().parent.parent)
    path = str(tmp_path / "forced.npz")
    code = _FORCED.format(root=root, shapes=shapes, path=path)
    envv = dict(os.environ, **env)
    envv["PYTHONPATH"] = str(Path(__file__).resolve().parent) + os.pathsep + envv.get("PYTHONPATH", "")
    subprocess.run([sys.executable, "-c", code], check=True, env=envv, timeout=600)
    z = np.load(path)
    for shape in shapes:
        A, b, _ = takagi(len(shape), 0.8, 1900 + sum(shape))
        assert rel(z["x".join(map(str, shape))], oracle_lib.vanilla(shape, A, b, 0.7 - 0.2j)) < FWD_TOL, (env, shape)


@pytest.mark.parametrize("shape", [(24,) * 4, (20, 20, 20), (16, 16, 16), (4096,), (8, 8, 8, 8)])
def test_stable_large_single(cuda, oracle_lib, shape):
    A, b, c = takagi(len(shape), 0.85, 204 + len(shape))
    G = mm.stable_numba(shape, A, b, c)
    assert rel(G, oracle_lib.stable(shape, A, b, c)) < FWD_TOL


def test_vjp_cfg4_vs_oracle(cuda, oracle_lib):
    A, b, c = takagi(4, 0.8, 303)
    shape = (30,) * 4
    G = oracle_lib.vanilla(shape, A, b, c)
    g = cn(shape, 304)
    ref = oracle_lib.vjp(G, c, g)
    got = mm.vanilla_vjp_numba(G, c, g)
    assert rel(got[0], ref[0]) < VJP_TOL
    assert rel(got[1], ref[1]) < VJP_TOL
    assert abs(got[2] - ref[2]) <= VJP_TOL * abs(ref[2])


def test_vjp_central_differences(cuda):
    """dA, db, dc vs central finite differences (h = 1e-6) of L = sum(dLdG * G) (holomorphic)."""
    A, b, c = takagi(3, 0.8, 305)
    c = 0.9 + 0.2j
    shape = (6, 5, 7)
    g = cn(shape, 306)
    G = mm.vanilla_numba(shape, A, b, c)
    dA, db, dc = mm.vanilla_vjp_numba(G, c, g)
    L = lambda A_, b_, c_: np.sum(g * mm.vanilla_numba(shape, A_, b_, c_))  # noqa: E731
    h = 1e-6
    for i in range(3):
        e = np.zeros(3)
        e[i] = h
        fd = (L(A, b + e, c) - L(A, b - e, c)) / (2 * h)
        assert abs(fd - db[i]) < 1e-6 * max(1, abs(fd))
        for j in range(3):
            E = np.zeros((3, 3))
            E[i, j] = h
            fdij = (L(A + E, b, c) - L(A - E, b, c)) / (2 * h)
            E = np.zeros((3, 3))
            E[j, i] = h
            fdji = (L(A + E, b, c) - L(A - E, b, c)) / (2 * h)
            assert abs((fdij + fdji) / 2 - dA[i, j]) < 1e-6 * max(1, abs(fdij))
    fdc = (L(A, b, c + h) - L(A, b, c - h)) / (2 * h)
    assert abs(fdc - dc) < 1e-6 * max(1, abs(fdc))


# ---------------------------------------------------------------- facade (test_vanilla.py:164-238)
def _rt(n, batch=(), seed=673):
    rng = np.random.RandomState(seed)
    A = rng.random((*batch, n, n)) + 1j * rng.random((*batch, n, n))
    A = A + np.swapaxes(A, -1, -2)
    A /= np.abs(np.linalg.eigvals(A)).max() + 0.2
    b = rng.random((*batch, n)) + 1j * rng.random((*batch, n))
    c = rng.random(batch) + 1j * rng.random(batch)
    return A, b, c


@pytest.mark.parametrize("stable", [True, False])
def test_facade_unbatched_and_out(cuda, stable):
    A, b, c = _rt(2)
    G = mm.hermite_renormalized(A, b, c, (3, 3), stable=stable)
    assert G.shape == (3, 3)
    out = np.zeros((3, 3), complex)
    G2 = mm.hermite_renormalized(A, b, c, (3, 3), stable=stable, out=out)
    assert G2 is out
    assert np.allclose(G2, G)


@pytest.mark.parametrize("stable", [True, False])
def test_facade_b_batched(cuda, stable):
    A, b, c = _rt(2, (2, 1))
    G = mm.hermite_renormalized(A[0, 0], b, c[0, 0], (4, 5), stable=stable)
    assert G.shape == (2, 1, 4, 5)
    assert np.allclose(G[0, 0], mm.hermite_renormalized(A[0, 0], b[0, 0], c[0, 0], (4, 5)))
    assert np.allclose(G[1, 0], mm.hermite_renormalized(A[0, 0], b[1, 0], c[0, 0], (4, 5)))
    out = np.zeros((2, 1, 4, 5), complex)
    G2 = mm.hermite_renormalized(A[0, 0], b, c[0, 0], (4, 5), stable=stable, out=out)
    assert np.allclose(G2, G) and np.allclose(out, G)


@pytest.mark.parametrize("stable", [True, False])
def test_facade_fully_batched(cuda, stable):
    A, b, c = _rt(2, (2, 1))
    G = mm.hermite_renormalized(A, b, c, (4, 5), stable=stable)
    assert G.shape == (2, 1, 4, 5)
    assert np.allclose(G[1, 0], mm.hermite_renormalized(A[1, 0], b[1, 0], c[1, 0], (4, 5)))
    out = np.zeros((2, 1, 4, 5), complex)
    mm.hermite_renormalized(A, b, c, (4, 5), stable=stable, out=out)
    assert np.allclose(out, G)


def test_device_tensors_stay_on_device(cuda, oracle_lib):
    A, b, c = takagi(3, 0.7, 401)
    At, bt = torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda)
    ct = torch.tensor(c, dtype=torch.complex128, device=cuda)
    G = mm.vanilla_numba((8, 9, 10), At, bt, ct)
    assert isinstance(G, torch.Tensor) and G.is_cuda
    assert rel(G, oracle_lib.vanilla((8, 9, 10), A, b, c)) < FWD_TOL
    out = torch.full((8, 9, 10), float("nan"), dtype=torch.complex128, device=cuda)
    G2 = mm.vanilla_numba((8, 9, 10), At, bt, ct, out=out)
    assert G2 is out and not torch.isnan(out).any()


def test_device_api_converts_dtypes(cuda, oracle_lib):
    """complex64 / real inputs to the device API are converted to complex128, not reinterpreted."""
    A, b, _ = takagi(2, 0.6, 950)
    G = mm.device_fwd(torch.as_tensor(A, device=cuda).to(torch.complex64).to(torch.complex128),
                      torch.as_tensor(b, device=cuda), torch.tensor(0.5 + 0.25j, device=cuda), (5, 6))
    ref = oracle_lib.vanilla((5, 6), A.astype(np.complex64).astype(complex), b, 0.5 + 0.25j)
    assert rel(G, ref) < FWD_TOL
    G2 = mm.device_fwd(torch.as_tensor(A.real, device=cuda), torch.as_tensor(b.real, device=cuda),
                       torch.tensor(2.0, device=cuda), (4, 4))
    assert rel(G2, oracle_lib.vanilla((4, 4), A.real, b.real, 2.0)) < FWD_TOL


def test_poisoned_output_fully_overwritten(cuda, oracle_lib):
    for D, shape in [(1, (9,)), (2, (1, 6)), (3, (4, 1, 5)), (4, (3, 4, 2, 5))]:
        A, b, c = takagi(D, 0.7, 500 + D)
        for stable in (False, True):
            out = torch.full(shape, complex(float("nan"), float("nan")), dtype=torch.complex128, device=cuda)
            mm.device_fwd(torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda),
                          torch.tensor(c, dtype=torch.complex128, device=cuda), shape, stable, out=out)
            assert not torch.isnan(out).any()
            ref = (oracle_lib.stable if stable else oracle_lib.vanilla)(shape, A, b, c)
            assert rel(out, ref) < FWD_TOL


@pytest.mark.parametrize("D", [5, 6, 7, 8])
def test_many_modes(cuda, oracle_lib, D):
    A, b, c = takagi(D, 0.8, 600 + D)
    shape = tuple([3, 2, 4, 2, 3, 2, 2, 3][:D])
    assert rel(mm.vanilla_numba(shape, A, b, c), oracle_lib.vanilla(shape, A, b, c)) < FWD_TOL
    assert rel(mm.stable_numba(shape, A, b, c), oracle_lib.stable(shape, A, b, c)) < FWD_TOL
    G = oracle_lib.vanilla(shape, A, b, c)
    g = cn(shape, 700 + D)
    ref = oracle_lib.vjp(G, c, g)
    got = mm.vanilla_vjp_numba(G, c, g)
    assert rel(got[0], ref[0]) < VJP_TOL and rel(got[1], ref[1]) < VJP_TOL


def test_too_many_modes_raises(cuda):
    with pytest.raises(_lib.MMError, match="UNSUPPORTED"):
        mm.vanilla_numba((2,) * 9, np.zeros((9, 9)), np.zeros(9), 1.0)


# ---------------------------------------------------------------- ragged batch
def _ragged_case(n, seed, cmax=12):
    rng = np.random.default_rng(seed)
    shapes, As, bs = [], [], []
    for k in range(n):
        D = int(rng.integers(1, 5))
        shapes.append(tuple(int(x) for x in rng.integers(1, cmax + 1, D)))
        A, b, _ = takagi(D, 0.8, seed * 100000 + k)
        As.append(A)
        bs.append(b)
    cs = np.exp(1j * rng.uniform(0, 2 * np.pi, n)) * rng.uniform(0.5, 1.0, n)
    return shapes, As, bs, cs


def test_ragged_forward_vjp_parity(cuda, oracle_lib):
    shapes, As, bs, cs = _ragged_case(300, 7)
    rb = mm.RaggedBatch(shapes)
    A, b, c = rb.pack(As, bs, cs)
    for stable in (False, True):
        G = rb.forward(A, b, c, stable=stable).cpu().numpy()
        for k, Gk in enumerate(rb.unpack(G)):
            ref = (oracle_lib.stable if stable else oracle_lib.vanilla)(shapes[k], As[k], bs[k], cs[k])
            assert rel(Gk, ref) < FWD_TOL, (k, shapes[k], stable)
    G = rb.forward(A, b, c)
    g = torch.as_tensor(cn(rb.total, 9), device=cuda)
    dA, db, dc = rb.vjp(G, c, g)
    dAs, dbs = rb.unpack_grads(dA.cpu().numpy(), db.cpu().numpy())
    Gs, gs = rb.unpack(G.cpu().numpy()), rb.unpack(g.cpu().numpy())
    dc = dc.cpu().numpy()
    for k in range(len(shapes)):
        rA, rb_, rc = oracle_lib.vjp(Gs[k], cs[k], gs[k])
        assert rel(dAs[k], rA) < VJP_TOL, k
        assert rel(dbs[k], rb_) < VJP_TOL, k
        assert abs(dc[k] - rc) <= VJP_TOL * max(1.0, abs(rc)), k


def test_ragged_graph_replay(cuda, oracle_lib):
    shapes, As, bs, cs = _ragged_case(64, 11, cmax=10)
    rb = mm.RaggedBatch(shapes)
    A, b, c = rb.pack(As, bs, cs)
    g = torch.as_tensor(cn(rb.total, 12), device=cuda)
    graph, G, (dA, db, dc) = rb.capture(A, b, c, g)
    G_e = rb.forward(A, b, c).clone()
    grads_e = [t.clone() for t in rb.vjp(G_e, c, g)]
    A2, b2, c2 = rb.pack([a * 0.9 for a in As], [x * 1.1 for x in bs], cs)
    A.copy_(A2)
    b.copy_(b2)
    graph.replay()
    torch.cuda.synchronize()
    for k, Gk in enumerate(rb.unpack(G.cpu().numpy())):
        assert rel(Gk, oracle_lib.vanilla(shapes[k], As[k] * 0.9, bs[k] * 1.1, cs[k])) < FWD_TOL
    A.copy_(rb.pack(As, bs, cs)[0])
    b.copy_(rb.pack(As, bs, cs)[1])
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(G, G_e)
    for t, e in zip((dA, db, dc), grads_e):
        assert torch.equal(t, e)  # deterministic reductions: bitwise reproducible


def test_ragged_shards_reproduce_unsharded_batch(cuda, oracle_lib):
    """RaggedBatch.shard: the shares of 3 ranks (run one after the other on this GPU; no rank waits
    on another) hold every instance once, and their G and gradients equal the unsharded batch's
    instance by instance (the forward bit for bit; the VJP within tolerance of the oracle)."""
    shapes, As, bs, cs = _ragged_case(90, 17, cmax=14)
    full = mm.RaggedBatch(shapes)
    A, b, c = full.pack(As, bs, cs)
    g_full = torch.as_tensor(cn(full.total, 18), device=cuda)
    G_full = full.forward(A, b, c)
    Gs_full = full.unpack(G_full.cpu().numpy())
    gs_full = full.unpack(g_full.cpu().numpy())
    seen = []
    for rank in range(3):
        rb = mm.RaggedBatch.shard(shapes, rank, 3)
        idx = list(rb.global_index)
        seen += idx
        Al, bl, cl = rb.pack([As[k] for k in idx], [bs[k] for k in idx], cs[idx])
        gl = torch.as_tensor(np.concatenate([gs_full[k].ravel() for k in idx]), device=cuda)
        Gl = rb.forward(Al, bl, cl)
        dA, db, dc = rb.vjp(Gl, cl, gl)
        dAs, dbs = rb.unpack_grads(dA.cpu().numpy(), db.cpu().numpy())
        for j, (k, Gk) in enumerate(zip(idx, rb.unpack(Gl.cpu().numpy()))):
            assert np.array_equal(Gk, Gs_full[k]), (rank, k)
            rA, rbb, rc = oracle_lib.vjp(Gs_full[k], cs[k], gs_full[k])
            assert rel(dAs[j], rA) < VJP_TOL and rel(dbs[j], rbb) < VJP_TOL, (rank, k)
            assert abs(dc.cpu().numpy()[j] - rc) <= VJP_TOL * max(1.0, abs(rc))
    assert sorted(seen) == list(range(len(shapes)))


# ---------------------------------------------------------------- autograd
def test_autograd_matches_finite_differences(cuda):
    A, b, _ = takagi(3, 0.7, 801)
    c = 0.8 + 0.1j
    shape = (7, 6, 5)
    T = torch.as_tensor(cn(shape, 802), device=cuda)
    T = T / T.abs().pow(2).sum().sqrt()

    def loss(A_, b_, c_):
        G = mm.hermite_renormalized_autograd(A_, b_, c_, shape)
        ov = (T.conj() * G).sum()
        return 1 - ov.abs() ** 2 / (G.abs() ** 2).sum()

    At = torch.tensor(A, device=cuda, requires_grad=True)
    bt = torch.tensor(b, device=cuda, requires_grad=True)
    ct = torch.tensor(c, dtype=torch.complex128, device=cuda, requires_grad=True)
    loss(At, bt, ct).backward()
    h = 1e-6
    with torch.no_grad():
        for i in range(3):
            for part in (1.0, 1j):
                e = torch.zeros(3, dtype=torch.complex128, device=cuda)
                e[i] = h * part
                fd = (loss(At, bt + e, ct) - loss(At, bt - e, ct)).item() / (2 * h)
                got = bt.grad[i].real if part == 1.0 else bt.grad[i].imag
                assert abs(fd - got.item()) < 1e-6
            E = torch.zeros(3, 3, dtype=torch.complex128, device=cuda)
            E[i, (i + 1) % 3] = h
            E[(i + 1) % 3, i] = h
            fd = (loss(At + E, bt, ct) - loss(At - E, bt, ct)).item() / (2 * h)
            got = (At.grad[i, (i + 1) % 3] + At.grad[(i + 1) % 3, i]).real.item()
            assert abs(fd - got) < 1e-6
        fd = (loss(At, bt, ct + h) - loss(At, bt, ct - h)).item() / (2 * h)
        assert abs(fd - ct.grad.real.item()) < 1e-6


# ---------------------------------------------------------------- failure handling
def test_bounded_wait_times_out_without_fault(cuda):
    """A grid barrier that can never complete gives up after its budget and records
    MM_ERR_WAIT_TIMEOUT in the workspace status word; the context stays usable."""
    lib = _lib.load()
    ws = torch.zeros(4096, dtype=torch.uint8, device=cuda)
    st = torch.cuda.current_stream().cuda_stream
    assert lib.mm_workspace_init(ws.data_ptr(), 4096, st) == 0
    assert lib.mm_test_wait_timeout(ws.data_ptr(), 4096, 20_000_000, st) == 0
    status = ctypes.c_int(-1)
    assert lib.mm_workspace_status(ws.data_ptr(), st, ctypes.byref(status)) == 0
    assert status.value == 5
    G = mm.vanilla_numba((5, 5), np.eye(2) * 0.1, np.ones(2) * 0.2, 1.0)  # still works
    assert np.isfinite(G).all()


def test_launch_count_increments(cuda):
    n0 = mm.launch_count()
    mm.vanilla_numba((4, 4), np.eye(2) * 0.1, np.ones(2) * 0.2, 1.0)
    assert mm.launch_count() >= n0 + 2


def test_ragged_step_host_matches_device(cuda, oracle_lib):
    """The host-buffer step (cotangent prefetched, read from pinned host memory, or uploaded in
    instance chunks whose VJPs start as they arrive; G copied back while the VJP runs) gives the
    same bits as the device-resident forward + VJP."""
    shapes, As, bs, cs = _ragged_case(48, 21, cmax=9)
    rb = mm.RaggedBatch(shapes)
    A, b, c = rb.pack(As, bs, cs)
    g = torch.as_tensor(cn(rb.total, 22), device=cuda)
    G_ref = rb.forward(A, b, c).clone()
    ref = [t.clone() for t in rb.vjp(G_ref, c, g)]
    pin = lambda t: t.cpu().pin_memory()  # noqa: E731
    A_h, b_h, c_h, g_h = pin(A), pin(b), pin(c), pin(g)
    G_h = torch.empty(rb.total, dtype=torch.complex128).pin_memory()
    outs = [torch.empty(n, dtype=torch.complex128).pin_memory() for n in (rb.n_a, rb.n_b, rb.B)]
    for mode, chunks in (("prefetch", 2), ("zero_copy", 2), ("pipelined", 2), ("pipelined", 3), ("prefetch", 2),
                         ("pipelined", 5), ("fused", 2), ("zero_copy", 2), ("fused", 2)):
        for o in (G_h, *outs):
            o.fill_(float("nan"))
        rb.step_host(A_h, b_h, c_h, g_h, G_h, *outs, cotangent=mode, chunks=chunks)
        torch.cuda.synchronize()
        assert torch.equal(G_h, G_ref.cpu()), mode
        for o, r in zip(outs, ref):
            assert torch.equal(o, r.cpu()), (mode, chunks)
    # the host copy of G split between the forward (instances k % 8 < s) and the VJP
    for split in (3, 8, 1, 0):
        for o in (G_h, *outs):
            o.fill_(float("nan"))
        rb.step_host(A_h, b_h, c_h, g_h, G_h, *outs, cotangent="fused", copy_split=split)
        torch.cuda.synchronize()
        assert torch.equal(G_h, G_ref.cpu()), split
        for o, r in zip(outs, ref):
            assert torch.equal(o, r.cpu()), split


def test_ragged_schedules_agree(cuda, oracle_lib):
    """Every schedule (cluster teams of 1..16 CTAs, thresholds, VJP item sizes) gives the same
    forward bits and a VJP within tolerance of the oracle; the autotuner picks one of them."""
    shapes, As, bs, cs = _ragged_case(40, 31, cmax=16)
    rb = mm.RaggedBatch(shapes)
    A, b, c = rb.pack(As, bs, cs)
    g = torch.as_tensor(cn(rb.total, 32), device=cuda)
    G0 = rb.forward(A, b, c).clone()
    for cl, tm in ((1, 0), (2, 64), (4, 256), (8, 1000), (16, 500)):
        try:
            rb.retune(team_min_amps=tm, team_cluster=cl)
        except _lib.MMError:
            continue
        assert torch.equal(rb.forward(A, b, c), G0), (cl, tm)
    Gs, gs = rb.unpack(G0.cpu().numpy()), rb.unpack(g.cpu().numpy())
    for it in (256, 4096, 1 << 16):
        rb.retune(vjp_item_amps=it)
        dA, db, dc = rb.vjp(G0, c, g)
        dAs, dbs = rb.unpack_grads(dA.cpu().numpy(), db.cpu().numpy())
        for k in range(0, len(shapes), 7):
            rA, rbb, _ = oracle_lib.vjp(Gs[k], cs[k], gs[k])
            assert rel(dAs[k], rA) < VJP_TOL and rel(dbs[k], rbb) < VJP_TOL
    choice = mm.autotune(rb, A, b, c, g, reps=1, use_cache=False)
    assert choice["team_cluster"] in (4, 8, 16) and choice["vjp_item_amps"] > 0
    assert torch.equal(rb.forward(A, b, c), G0)


def test_cfg4_gradient_d4_cutoff30(cuda, oracle_lib):
    """4-mode triple at cutoff 30: dA, db, dc vs central differences (h = 1e-6, real
    perturbations, holomorphic) of L = sum(dLdG * G) and vs the oracle's vanilla_vjp."""
    A, b, c = takagi(4, 0.8, 1401)
    c = 0.9 - 0.2j
    shape = (30,) * 4
    g = cn(shape, 1402)
    At, bt = torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda)
    ct = torch.tensor(c, dtype=torch.complex128, device=cuda)
    gt = torch.as_tensor(g, device=cuda)
    G = mm.device_fwd(At, bt, ct, shape)
    dA, db, dc = (x.cpu().numpy() for x in mm.device_vjp(G, ct, gt, batched=False))
    rA, rb_, rc = oracle_lib.vjp(G.cpu().numpy(), c, g)
    assert rel(dA, rA) < VJP_TOL and rel(db, rb_) < VJP_TOL and abs(dc - rc) <= VJP_TOL * abs(rc)

    def L(A_, b_, c_):
        Gx = mm.device_fwd(torch.as_tensor(A_, device=cuda), torch.as_tensor(b_, device=cuda),
                           torch.tensor(c_, dtype=torch.complex128, device=cuda), shape)
        return complex((gt * Gx).sum().item())

    h = 1e-6
    scale = max(np.abs(dA).max(), np.abs(db).max())
    for i in range(4):
        e = np.zeros(4)
        e[i] = h
        fd = (L(A, b + e, c) - L(A, b - e, c)) / (2 * h)
        assert abs(fd - db[i]) < 1e-6 * scale
        j = (i + 1) % 4
        E = np.zeros((4, 4))
        E[i, j] = E[j, i] = h
        fd = (L(A + E, b, c) - L(A - E, b, c)) / (2 * h)  # symmetric perturbation = dA_ij + dA_ji
        assert abs(fd - 2 * dA[i, j]) < 1e-6 * scale
    fd = (L(A, b, c + h) - L(A, b, c - h)) / (2 * h)
    assert abs(fd - dc) < 1e-6 * max(1.0, abs(dc))


def test_cfg4_batched_fidelity_step(cuda):
    """64-instance batched gradient step: loss = sum_k 1 - |<T, G_k>|^2 / <G_k, G_k> with a fixed
    random normalised target T; autograd gradients vs central differences on sampled entries."""
    B, shape = 64, (30,) * 4
    trip = [takagi(4, 0.8, 1500 + k) for k in range(B)]
    A = torch.as_tensor(np.stack([t[0] for t in trip]), device=cuda).requires_grad_(True)
    b = torch.as_tensor(np.stack([t[1] for t in trip]), device=cuda).requires_grad_(True)
    c = torch.ones(B, dtype=torch.complex128, device=cuda, requires_grad=True)
    T = torch.as_tensor(cn(shape, 1600), device=cuda)
    T = T / T.abs().pow(2).sum().sqrt()

    def loss(A_, b_, c_):
        G = mm.hermite_renormalized_autograd(A_, b_, c_, shape)  # (B, 30, 30, 30, 30)
        ov = (T.conj() * G).sum(dim=(1, 2, 3, 4))
        return (1 - ov.abs() ** 2 / G.abs().pow(2).sum(dim=(1, 2, 3, 4))).sum()

    l0 = loss(A, b, c)
    l0.backward()
    assert torch.isfinite(A.grad).all() and torch.isfinite(b.grad).all()
    h = 1e-6
    with torch.no_grad():
        for k, i in ((0, 0), (17, 2), (63, 3)):
            for part in (1.0, 1j):
                e = torch.zeros_like(b)
                e[k, i] = h * part
                fd = (loss(A, b + e, c) - loss(A, b - e, c)).item() / (2 * h)
                got = b.grad[k, i].real if part == 1.0 else b.grad[k, i].imag
                assert abs(fd - got.item()) < 1e-6
            j = (i + 1) % 4
            E = torch.zeros_like(A)
            E[k, i, j] = E[k, j, i] = h
            fd = (loss(A + E, b, c) - loss(A - E, b, c)).item() / (2 * h)
            assert abs(fd - (A.grad[k, i, j] + A.grad[k, j, i]).real.item()) < 1e-6


@pytest.mark.parametrize("shape", [(20, 20, 20), (6, 5, 7), (30, 30, 30, 30), (4097,)])
def test_host_buffer_entry_points_match_device(cuda, shape):
    """mm_hermite_fwd_host / mm_hermite_vjp_host (numpy in, numpy out, staged through the library's
    own pinned and device buffers) give the same bits as the device-tensor calls, into a caller's
    `out` too (the reference returns `out` itself, test_vanilla.py:177-186)."""
    D = len(shape)
    A, b, c = takagi(D, 0.8, 1700 + D)
    for stable in (False, True):
        G_host = (mm.stable_numba if stable else mm.vanilla_numba)(shape, A, b, c)
        G_dev = mm.device_fwd(torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda),
                              torch.tensor(c, dtype=torch.complex128, device=cuda), shape, stable).cpu().numpy()
        assert isinstance(G_host, np.ndarray) and G_host.shape == shape
        assert np.array_equal(G_host, G_dev), stable
        out = np.empty(shape, np.complex128)
        assert (mm.stable_numba if stable else mm.vanilla_numba)(shape, A, b, c, out=out) is out
        assert np.array_equal(out, G_dev)
    g = cn(shape, 1701)
    dA, db, dc = mm.vanilla_vjp_numba(G_host, c, g)
    dA_d, db_d, dc_d = mm.device_vjp(torch.as_tensor(G_host, device=cuda), torch.tensor(c, dtype=torch.complex128,
                                     device=cuda), torch.as_tensor(g, device=cuda), batched=False)
    assert np.array_equal(dA, dA_d.cpu().numpy()) and np.array_equal(db, db_d.cpu().numpy())
    assert dc == complex(dc_d.item())


def test_empty_batches(cuda):
    """A batch of zero triples (the reference's loop over an empty batch axis, batch.py:52-61 and
    gradients.py:85-116) gives empty outputs of the reference's shapes."""
    A = np.zeros((0, 2, 2), np.complex128)
    b = np.zeros((0, 2), np.complex128)
    c = np.zeros((0,), np.complex128)
    G = mm.vanilla_batch_numba((3, 4), A, b, c)
    assert G.shape == (0, 3, 4) and G.dtype == np.complex128
    dA, db, dc = mm.vanilla_batch_vjp_numba(G, c, np.zeros((0, 3, 4), np.complex128))
    assert dA.shape == (0, 2, 2) and db.shape == (0, 2) and dc.shape == (0,)
