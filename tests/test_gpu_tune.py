"""The autotuner changes launch shapes only: results with tuned and heuristic
tiles are bit-identical (3D periodic FFT passes, 2D Dirichlet dense passes in
FP64, both precisions), and so are the fused 2D loop's tuned and heuristic
launch forms."""
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


@pytest.mark.parametrize("B", [2, 40])
def test_autotune_invariant_fused_loop(srn, B):
    """The fused FP32 2D loop (tensor-core z tail) with its launch form timed at
    context creation against the heuristic form: the same records and fields,
    bit for bit, for a batch below and one above one chain per SM."""
    s = srn.configs.film2d(nx=192, nz=96, ns=40, iters=3)
    w = srn.configs.droplet_fields(s, seed=5)
    m = srn.configs.substrate_mask(s)

    def run(tune):
        with srn.Solver([s.copy() for _ in range(B)], precision="fp32", autotune=tune) as sv:
            tpl = sv.timing()["threads_per_line"]
            for b in range(B):
                sv.set_fields(w, b)
                sv.set_masks(m, b)
                sv.set_iteration(1, b)
            out = sv.iterate(3)
            return tpl, [o[B - 1].free_energy for o in out], sv.get_fields(B - 1)

    ta, fa, wa = run(True)
    tb, fb, wb = run(False)
    assert ta in (1, 2) and tb in (1, 2)
    assert fa == fb
    np.testing.assert_array_equal(wa, wb)

