"""CPU-side checks of the C ABI: the library builds, loads, exports every declared symbol,
and its host-only entry points (sizes, planning, status text) behave; no kernel runs here."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from mrmustard_gb300 import _lib


def test_library_exports_every_header_symbol():
    lib = _lib.load()
    declared = _lib.header_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) <= set(_lib.SIGNATURES), set(declared) - set(_lib.SIGNATURES)


def test_status_strings_and_limits():
    lib = _lib.load()
    assert lib.mm_status_string(0) == b"ok"
    assert b"timed out" in lib.mm_status_string(5)
    assert lib.mm_max_modes() == 8


def test_workspace_size_is_host_only():
    lib = _lib.load()
    sh = (ctypes.c_int64 * 4)(40, 40, 40, 40)
    n1 = lib.mm_hermite_workspace_bytes(4, sh, 1)
    n64 = lib.mm_hermite_workspace_bytes(4, sh, 64)
    assert n1 > 512 and n64 > n1
    bad = (ctypes.c_int64 * 2)(3, 0)
    assert lib.mm_hermite_workspace_bytes(2, bad, 1) == 0  # shape entry 0 is rejected
    assert lib.mm_hermite_workspace_bytes(9, (ctypes.c_int64 * 9)(*[2] * 9), 1) == 0  # D > 8


def test_ragged_plan_on_host():
    lib = _lib.load()
    shapes = [(3, 4), (5,), (2, 2, 2), (7, 1, 3, 2)]
    D = np.array([len(s) for s in shapes], np.int32)
    flat = np.array([x for s in shapes for x in s], np.int64)
    plan = ctypes.c_void_p()
    assert lib.mm_ragged_plan_create(len(shapes), D.ctypes.data, flat.ctypes.data, ctypes.byref(plan)) == 0
    try:
        assert lib.mm_ragged_plan_amplitudes(plan) == 12 + 5 + 8 + 42
        g = np.zeros(4, np.int64)
        a = np.zeros(4, np.int64)
        b = np.zeros(4, np.int64)
        assert lib.mm_ragged_plan_offsets(plan, g.ctypes.data, a.ctypes.data, b.ctypes.data) == 0
        assert list(g) == [0, 12, 17, 25]
        assert list(a) == [0, 4, 5, 14]
        assert list(b) == [0, 2, 3, 6]
        assert lib.mm_ragged_plan_workspace_bytes(plan) > 512
        assert lib.mm_ragged_plan_set_tuning(plan, 0, 1000) == 0
        assert lib.mm_ragged_plan_set_tuning(plan, -1, 1000) == 1
        # split of the host copy of G between forward and VJP: eighths 0..8
        for s in (0, 2, 8):
            assert lib.mm_ragged_plan_set_copy_split(plan, s) == 0
        assert lib.mm_ragged_plan_set_copy_split(plan, 9) == 1
        assert lib.mm_ragged_plan_set_copy_split(plan, -1) == 1
    finally:
        lib.mm_ragged_plan_destroy(plan)
    bad = np.array([2, 0], np.int64)
    plan2 = ctypes.c_void_p()
    assert lib.mm_ragged_plan_create(1, np.array([2], np.int32).ctypes.data, bad.ctypes.data,
                                     ctypes.byref(plan2)) == 1


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-device path")
def test_compute_entry_reports_no_device():
    lib = _lib.load()
    sh = (ctypes.c_int64 * 1)(4)
    rc = lib.mm_hermite_fwd(1, sh, None, None, None, 0, None, None, 0, None)
    assert rc == 7  # MM_ERR_NO_DEVICE: there is no CPU path


def test_product_refuses_cpu():
    import mrmustard_gb300 as mm

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(RuntimeError, match="CUDA device"):
        mm.vanilla((3, 3), np.zeros((2, 2)), np.zeros(2), 1.0)
