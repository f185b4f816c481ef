"""scft_propagate_static: the propagator entry point for callers that cannot
allocate device memory at run time (its working buffers sit in one fixed
device array). Checked through the C ABI against scft_propagate on two calls in
a row, at the tolerance of the propagator parity tests (1e-11 relative).

This file is collected last on purpose: the entry point keeps state (the fixed
array and its per-device address) for the life of the process.
"""
import ctypes as C
import importlib

import numpy as np
import pytest

from conftest import load_golden, surface_from_json

pytestmark = pytest.mark.gpu


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.parametrize("tag,precision", [("periodic2d", "fp64"), ("dirichlet2d", "fp64"), ("periodic3d", "fp64"),
                                           ("dirichlet2d", "fp32")])
def test_static_matches_allocating_entry_point(tag, precision, srn):
    L = importlib.import_module("stimuli-responsive-nanodroplets_gb300._lib")
    lib = L.lib()
    g = load_golden(f"kat_prop_{tag}")
    S = surface_from_json(srn, g["surface"])
    steps = g["q"].shape[0] - 1
    rng = np.random.default_rng(7)
    with srn.Solver(S, precision=precision) as sv:
        M = sv.M
        for call in range(2):  # two calls in a row: the array keeps the last call's data
            q0 = np.ascontiguousarray(g["q0"] if call == 0 else 1.0 + 0.1 * rng.standard_normal(M))
            w = np.ascontiguousarray(g["w"] if call == 0 else 0.3 * rng.standard_normal(M))
            want = np.empty((steps + 1, M))
            got = np.empty((steps + 1, M))
            L.check(lib.scft_propagate(sv._h, _dp(q0), _dp(w), steps, _dp(want)), "scft_propagate")
            L.check(lib.scft_propagate_static(sv._h, _dp(q0), _dp(w), steps, _dp(got)), "scft_propagate_static")
            np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-13)
            if call == 0 and precision == "fp64":
                np.testing.assert_allclose(got, g["q"], rtol=1e-11, atol=1e-13)


def test_static_rejects_oversized_requests(srn):
    L = importlib.import_module("stimuli-responsive-nanodroplets_gb300._lib")
    lib = L.lib()
    cap = lib.scft_static_scratch_bytes()
    S = srn.configs.film2d(iters=1)
    with srn.Solver(S, precision="fp64") as sv:
        M = sv.M
        steps = int(cap // (M * 16)) + 10
        q0 = np.ones(M)
        w = np.zeros(M)
        out = np.empty((steps + 1, M))
        rc = lib.scft_propagate_static(sv._h, _dp(q0), _dp(w), steps, _dp(out))
        assert rc == -1
        assert b"fixed" in lib.scft_last_error()


def test_static_call_allocates_no_device_memory(srn):
    """The defining property: once the array's address is known (first call),
    a call leaves the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    L = importlib.import_module("stimuli-responsive-nanodroplets_gb300._lib")
    lib = L.lib()
    g = load_golden("kat_prop_dirichlet2d")
    S = surface_from_json(srn, g["surface"])
    steps = g["q"].shape[0] - 1
    with srn.Solver(S, precision="fp32") as sv:
        q0 = np.ascontiguousarray(g["q0"])
        w = np.ascontiguousarray(g["w"])
        out = np.empty((steps + 1, sv.M))
        L.check(lib.scft_propagate_static(sv._h, _dp(q0), _dp(w), steps, _dp(out)), "scft_propagate_static")
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        for _ in range(3):
            L.check(lib.scft_propagate_static(sv._h, _dp(q0), _dp(w), steps, _dp(out)), "scft_propagate_static")
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
    assert abs(free1 - free0) <= (2 << 20)

