"""The 64^3 cluster-resident contour loop (FP32, MASK 0) against the FP64
plain form, against the FP32 per-axis passes, and directly against the
reference's own series of the four-diblock blend at 64^3."""
import importlib

import numpy as np
import pytest

from conftest import load_golden, surface_from_json

pytestmark = pytest.mark.gpu


def _bulk(srn, ns=40):
    return srn.configs.bulk3d_point(18.0, 36.0, srn.configs.PLANES[0], n=64, ns=ns)


def test_fused3d_is_used_and_propagates_like_fp64(srn):
    s = _bulk(srn)
    M = 64 ** 3
    rng = np.random.default_rng(5)
    q0 = rng.uniform(0.5, 1.5, M)
    w = rng.uniform(-0.5, 0.5, M)
    with srn.Solver(s, precision="fp32") as sv:
        sv.enable_timing(True)
        sv.set_fields(np.zeros((14, M)))
        sv.set_iteration(1)
        sv.iterate(1)
        assert sv.timing()["fused_chain"] == 2
        q32 = sv.propagate(q0, w, 20)
    with srn.Solver(s, precision="fp32", kernel_path="passes") as sv:
        q32p = sv.propagate(q0, w, 20)
    with srn.Solver(s, precision="fp64") as sv:
        q64 = sv.propagate(q0, w, 20)
    scale = np.abs(q64).max(axis=1, keepdims=True)
    err = np.abs(q32 - q64) / scale
    errp = np.abs(q32p - q64) / scale
    assert err.max() < 3e-6, err.max()
    # the cluster kernel is at least as accurate as the FP32 passes (to within a factor)
    assert err.max() < 3.0 * errp.max() + 1e-7, (err.max(), errp.max())


def test_fused3d_iterations_vs_fp64_and_batch(srn):
    s = _bulk(srn)
    w = srn.configs.seed_fields(s, "lamellar", seed=4)
    res = {}
    for prec in ("fp32", "fp64"):
        with srn.Solver([s, s.copy()], precision=prec) as sv:
            for b in range(2):
                sv.set_fields(w, b)
                sv.set_iteration(1, b)
            out = sv.iterate(3)
            res[prec] = (out, sv.get_fields(1))
    for k in range(3):
        f32, f64 = res["fp32"][0][k][1].free_energy, res["fp64"][0][k][1].free_energy
        assert abs(f32 - f64) <= 3e-6 * abs(f64), (k, f32, f64)
        assert res["fp32"][0][k][0].free_energy == res["fp32"][0][k][1].free_energy
    with srn.Solver(s, precision="fp32") as solo:
        solo.set_fields(w)
        solo.set_iteration(1)
        o = solo.iterate(3)
        assert o[-1][0].free_energy == res["fp32"][0][-1][1].free_energy
        np.testing.assert_array_equal(solo.get_fields(), res["fp32"][1])


def test_fused3d_against_reference_series(srn):
    """The four-diblock blend of the third configuration (64^3, NS 128, 11
    chains, noise from the drand48 replay) through the cluster kernel: it runs
    the fused loop, and every iteration's free energy is within 3e-6 of the
    reference's own (tests/golden/blend3d_full, SCFT.c on the same start)."""
    g = load_golden("blend3d_full")
    S = surface_from_json(srn, g["surface"])
    w0 = srn.configs.uniform_fields(S.grid(), seed=1000, amp=0.1, fields=tuple(range(9)))
    np.testing.assert_allclose(w0.sum(axis=1), g["w_sum"], rtol=0, atol=1e-9)
    runner = importlib.import_module("stimuli-responsive-nanodroplets_gb300.runner")
    r = runner.Run(S, w0, int(g["counter"]), tuple(int(x) for x in g["seed0"]), None, precision="fp32",
                   noise="device")
    r.solver.enable_timing(True)
    r.run_to_end()
    assert r.solver.timing()["fused_chain"] == 2
    by_iter = {rec.iter: rec for rec in r.records}
    for row in g["free_energy"]:
        got = by_iter[int(row[0])].free_energy
        assert abs(got - row[1]) <= 3e-6 * abs(row[1]), (row[0], got, row[1])

