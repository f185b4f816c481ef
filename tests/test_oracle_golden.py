"""The CPU oracle against outputs of the reference solver itself (tests/golden).

These pin the oracle before it is trusted as the checker of the GPU library:
every golden case was produced by the unmodified SCFT.c (tests/golden/make_golden.py).
"""
import numpy as np
import pytest

CASES = ["bulk2d", "film2d", "blend3d", "quirks", "seed"]


def run_oracle(oracle_mod, g):
    """Run the oracle through the restart path; also track what the reference
    writes to restart_random.dat. At each snapshot SCFT.c calls seed48 twice
    (SCFT.c:1653-1657) and then prints through the pointer the first call
    returned, which the second call has overwritten: the file receives the
    state saved at the previous snapshot (the restart seed at the first one),
    while the running stream itself is restored correctly."""
    S = g["S"]
    o = oracle_mod.Oracle(S)
    counter = int(g["counter"])
    seed = tuple(int(x) for x in g["seed0"])
    if counter > 0:
        o.set_fields(g["w0"])
        o.set_rng(seed)
    o.set_masks(g["mask3"])
    o.set_iter(counter)
    n = int(S.ITER) - counter + 1  # iterations numbered counter+1 .. ITER+1 (SCFT.c:1088-1090)
    recs = []
    saved = seed
    written = None
    snap = int(g["snap_iter"])
    for _ in range(n):
        r = o.iterate(1)[0]
        recs.append(r)
        it = int(r[0])
        if it % int(S.D_WRT) == 0 or it == 1:
            written = saved
            saved = o.get_rng()
        if it == snap:
            o.snap_phi = o.densities()[0]
            o.snap_w = o.get_fields()
    o.rng_file = written
    return o, np.array(recs)


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference(case, golden, oracle_mod):
    g = golden(case)
    S = g["S"]
    o, rec = run_oracle(oracle_mod, g)
    fe = g["free_energy"]
    # free_energy.dat lines are written every D_WRT_ENERGIES iterations
    by_iter = {int(r[0]): r for r in rec}
    for row in fe:
        r = by_iter[int(row[0])]
        assert abs(r[1] - row[1]) <= 1e-12 * max(1.0, abs(row[1])), (case, row[0], r[1], row[1])
        assert r[3] == row[2]
    for row in g["energies"]:
        r = by_iter[int(row[0])]
        np.testing.assert_allclose(r[4:4 + 17], row[1:], rtol=1e-11, atol=1e-12)
    for row in g["deviations"]:
        r = by_iter[int(row[0])]
        assert abs(r[2] - row[1]) <= 1e-10 * max(1e-6, abs(row[1])) + 1e-15
    # the last snapshot (densities file + restart fields) of the run
    np.testing.assert_allclose(o.snap_phi, g["snap_phi"], rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(o.snap_w, g["snap_w"], rtol=1e-11, atol=1e-12)
    np.testing.assert_allclose(o.snap_w, g["restart_w"], rtol=1e-11, atol=1e-12)
    assert int(g["counter_out"]) == int(g["snap_iter"])
    if int(g["counter"]) > 0:
        assert o.rng_file == tuple(int(x) for x in g["restart_rng"])


@pytest.mark.parametrize("tag", ["periodic2d", "dirichlet2d", "periodic3d"])
def test_oracle_propagator_matches_funPDESolver(tag, srn, oracle_mod):
    from conftest import load_golden, surface_from_json
    g = load_golden(f"kat_prop_{tag}")
    S = surface_from_json(srn, g["surface"])
    o = oracle_mod.Oracle(S)
    q = o.propagate(g["q0"], g["w"], g["q"].shape[0] - 1)
    np.testing.assert_allclose(q, g["q"], rtol=1e-12, atol=1e-14)


def test_oracle_surface_layout_matches_library(srn, oracle_mod):
    import ctypes
    from importlib import import_module
    L = import_module("stimuli-responsive-nanodroplets_gb300._lib")
    assert oracle_mod.lib().orc_surface_size() == ctypes.sizeof(L.CSurface)


def test_oracle_density_matches_funDensity(srn, oracle_mod):
    """funMultiplyQs + funDensity of the reference (shared build, kat_density_2d)
    against the oracle's restatement, including the point stop-1 that an odd
    interval count leaves out."""
    from conftest import load_golden
    g = load_golden("kat_density_2d")
    nx, ny, nz = (int(v) for v in g["grid"])
    S = srn.configs.bulk2d(nx=nx, nz=nz, iters=1)
    o = oracle_mod.Oracle(S)
    for (start, stop), phi in zip(g["blocks"], g["phi"]):
        got = o.density(g["qf"], g["qb"], int(start), int(stop), float(g["Q"]))
        np.testing.assert_allclose(got, phi, rtol=1e-14, atol=0)
    o.close()
