"""The 64^3 cluster-resident contour loop (FP32, MASK 0) against the FP64
plain form and against the FP32 per-axis passes."""
import numpy as np
import pytest

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
