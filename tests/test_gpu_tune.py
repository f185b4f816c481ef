"""The pass-tile autotuner changes launch shapes only: results with tuned and
heuristic tiles are bit-identical (3D periodic FFT passes, 2D Dirichlet dense
passes in FP64, both precisions)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(srn, s, w, m, precision, autotune, kernel_path="auto", n=3):
    with srn.Solver([s, s.copy()], precision=precision, autotune=autotune, kernel_path=kernel_path) as sv:
        for b in range(2):
            sv.set_fields(w, b)
            if m is not None:
                sv.set_masks(m, b)
            sv.set_iteration(1, b)
        out = sv.iterate(n)
        return [o[1].free_energy for o in out], sv.get_fields(1)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_autotune_invariant_3d(srn, precision):
    s = srn.configs.bulk3d_point(18.0, 35.0, srn.configs.PLANES[0], n=16, ns=30)
    w = srn.configs.seed_fields(s, "lamellar", seed=3)
    a = _run(srn, s, w, None, precision, True)
    b = _run(srn, s, w, None, precision, False)
    assert a[0] == b[0]
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_autotune_invariant_film_passes(srn, precision):
    s = srn.configs.film2d(nx=48, nz=24, ns=40, iters=3)
    w = srn.configs.droplet_fields(s, seed=3, radius=2.0)
    m = srn.configs.substrate_mask(s)
    a = _run(srn, s, w, m, precision, True, kernel_path="passes")
    b = _run(srn, s, w, m, precision, False, kernel_path="passes")
    assert a[0] == b[0]
    np.testing.assert_array_equal(a[1], b[1])
