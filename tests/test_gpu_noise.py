"""Device replay of the drand48 noise stream against the reference (golden runs
with noise) and against the host replay, state by state."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def runner():
    return importlib.import_module("stimuli-responsive-nanodroplets_gb300.runner")


@pytest.mark.parametrize("case", ["blend3d", "quirks", "bulk2d"])
def test_device_noise_matches_reference(case, srn, golden):
    g = golden(case)
    r = runner().Run(g["S"], g["w0"], int(g["counter"]), tuple(int(x) for x in g["seed0"]), g["mask3"],
                     precision="fp64", noise="device")
    r.run_to_end(keep_snapshots=True)
    by_iter = {rec.iter: rec for rec in r.records}
    for row in g["free_energy"]:
        rec = by_iter[int(row[0])]
        assert abs(rec.free_energy - row[1]) <= 1e-9 * max(1.0, abs(row[1]))
    phi, w, written = r.snapshots[int(g["snap_iter"])]
    np.testing.assert_allclose(w, g["restart_w"], rtol=1e-10, atol=1e-10)
    assert written == tuple(int(x) for x in g["restart_rng"])


def test_device_state_matches_host_replay_every_iteration(srn):
    S = srn.configs.blend3d(n=16, ns=24, iters=4)
    S.RELAXATION = 2
    w = srn.configs.uniform_fields(S.grid(), seed=4, amp=0.1, fields=tuple(range(9)))
    d = srn.derive(S)
    seed = (101, 202, 303)
    with srn.Solver(S, precision="fp64", noise="device") as sv:
        sv.set_fields(w)
        sv.set_iteration(1)
        sv.set_rng(seed)
        state = seed
        for _ in range(4):
            sv.iterate(1)
            _, state = srn.noise_fill(state, d, out=False)
            assert sv.get_rng() == state
