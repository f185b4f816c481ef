"""The fused single-launch 2D contour step (FP32 form) against the per-axis
passes and against the reference's funPDESolver.

Tolerance: FP32 arithmetic over tens of contour steps, 2e-5 relative to the
slice maximum.
"""
import importlib

import numpy as np
import pytest

from conftest import load_golden, surface_from_json

pytestmark = pytest.mark.gpu
RTOL32 = 2e-5


@pytest.mark.parametrize("tag", ["periodic2d", "dirichlet2d"])
def test_fused_propagate_matches_funPDESolver(tag, srn):
    g = load_golden(f"kat_prop_{tag}")
    S = surface_from_json(srn, g["surface"])
    with srn.Solver(S, precision="fp32") as sv:
        q = sv.propagate(g["q0"], g["w"], g["q"].shape[0] - 1)
    scale = np.abs(g["q"]).max(axis=1, keepdims=True)
    assert np.all(np.abs(q - g["q"]) <= RTOL32 * scale)


@pytest.mark.parametrize("shape,mask", [((192, 96), 1), ((192, 128), 1), ((128, 96), 1), ((96, 64), 1),
                                        ((64, 64), 0), ((64, 32), 0), ((32, 32), 0), ((32, 24), 0),
                                        ((32, 16), 1), ((24, 16), 0), ((16, 16), 0)])
def test_fused_matches_axis_passes(shape, mask, srn):
    nx, nz = shape
    if mask:
        S = srn.configs.film2d(nx=nx, nz=nz, ns=64, iters=1)
    else:
        S = srn.configs.bulk2d(nx=nx, nz=nz, iters=1)
    rng = np.random.default_rng(nx * 1000 + nz)
    q0 = 1.0 + 0.3 * rng.standard_normal(nx * nz)
    w = 0.8 * rng.standard_normal(nx * nz)
    with srn.Solver(S, precision="fp32") as a, srn.Solver(S, precision="fp32", kernel_path="passes") as b, \
            srn.Solver(S, precision="fp64", kernel_path="passes") as c:
        qa = a.propagate(q0, w, 20)
        qb = b.propagate(q0, w, 20)
        qc = c.propagate(q0, w, 20)
    scale = np.abs(qc).max(axis=1, keepdims=True)
    assert np.all(np.abs(qa - qc) <= RTOL32 * scale)
    assert np.all(np.abs(qb - qc) <= RTOL32 * scale)


def test_fused_iterations_film(srn, golden):
    """Whole iterations with the fused step on the thin-film golden run: free
    energy within 1e-6 relative of the reference."""
    runner = importlib.import_module("stimuli-responsive-nanodroplets_gb300.runner")
    g = golden("film2d")
    r = runner.Run(g["S"], g["w0"], int(g["counter"]), tuple(int(x) for x in g["seed0"]), g["mask3"],
                   precision="fp32")
    r.run_to_end()
    by_iter = {rec.iter: rec for rec in r.records}
    for row in g["free_energy"]:
        assert abs(by_iter[int(row[0])].free_energy - row[1]) <= 1e-6 * max(1.0, abs(row[1]))


@pytest.mark.parametrize("nx,nz", [(192, 96), (192, 128), (128, 96), (96, 64), (64, 32)])
def test_two_threads_per_line_bit_identical(srn, nx, nz):
    """A batch of at most one chain per SM gives every line two threads; an
    instance must come out bit for bit as it does in a batch too large for
    that (one thread per line): records, fields and densities."""
    s = srn.configs.film2d(nx=nx, nz=nz, ns=40, iters=3)
    w = srn.configs.droplet_fields(s, seed=7, radius=nx * 0.125 / 5)
    m = srn.configs.substrate_mask(s)

    def run(B):
        # the heuristic form (autotune off): two threads per line exactly when
        # the batch has at most one chain per SM
        with srn.Solver([s] * B, precision="fp32", autotune=False) as sv:
            tpl = sv.timing()["threads_per_line"]
            for b in range(B):
                sv.set_fields(w, b)
                sv.set_masks(m, b)
                sv.set_iteration(1, b)
            out = sv.iterate(3)
            phi, tot = sv.get_densities(0)
            return tpl, [r[0] for r in out], sv.get_fields(0), phi, tot

    t1, o1, w1, p1, s1 = run(1)
    tb, ob, wb, pb, sb = run(40)          # 40 instances x 5 chains: more chains than SMs
    assert t1 == 2 and tb == 1
    for a, b in zip(o1, ob):
        assert a.free_energy == b.free_energy and a.rms == b.rms
        np.testing.assert_array_equal(a.q, b.q)
    np.testing.assert_array_equal(w1, wb)
    np.testing.assert_array_equal(p1, pb)
    np.testing.assert_array_equal(s1, sb)
