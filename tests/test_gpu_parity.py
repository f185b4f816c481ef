"""GPU parity: the CUDA library (FP64 plain form) against the reference's own
outputs (tests/golden) and the CPU oracle, through the C ABI.

Tolerances (the plain form's contract): densities 1e-10 relative, free energy
1e-9 relative per chain; propagator slices 1e-11.
"""
import importlib

import numpy as np
import pytest

from conftest import load_golden, surface_from_json

pytestmark = pytest.mark.gpu

CASES = ["bulk2d", "film2d", "blend3d", "quirks", "seed"]
PHI_RTOL = 1e-10
F_RTOL = 1e-9


def runner_mod():
    return importlib.import_module("stimuli-responsive-nanodroplets_gb300.runner")


def run_gpu(srn, g, precision="fp64", use_graph=False):
    S = g["S"]
    counter = int(g["counter"])
    r = runner_mod().Run(S, g["w0"] if counter > 0 else None, counter, tuple(int(x) for x in g["seed0"]),
                         g["mask3"], precision=precision, use_graph=use_graph)
    r.run_to_end(keep_snapshots=True)
    return r


@pytest.mark.parametrize("tag", ["periodic2d", "dirichlet2d", "periodic3d"])
def test_propagate_matches_funPDESolver(tag, srn):
    g = load_golden(f"kat_prop_{tag}")
    S = surface_from_json(srn, g["surface"])
    with srn.Solver(S, precision="fp64") as sv:
        q = sv.propagate(g["q0"], g["w"], g["q"].shape[0] - 1)
    np.testing.assert_allclose(q, g["q"], rtol=1e-11, atol=1e-13)


@pytest.mark.parametrize("case", CASES)
def test_iterations_match_reference(case, srn, golden):
    g = golden(case)
    r = run_gpu(srn, g)
    by_iter = {rec.iter: rec for rec in r.records}
    for row in g["free_energy"]:
        rec = by_iter[int(row[0])]
        assert abs(rec.free_energy - row[1]) <= F_RTOL * max(1.0, abs(row[1])), (case, row[0], rec.free_energy, row[1])
        assert rec.mf == row[2]
    for row in g["energies"]:
        rec = by_iter[int(row[0])]
        np.testing.assert_allclose(rec.mu, row[1:], rtol=1e-10, atol=1e-11)
    for row in g["deviations"]:
        rec = by_iter[int(row[0])]
        assert abs(rec.rms - row[1]) <= 1e-9 * abs(row[1]) + 1e-13
    phi, w, written = r.snapshots[int(g["snap_iter"])]
    scale = np.maximum(np.abs(g["snap_phi"]).max(axis=1, keepdims=True), 1e-300)
    assert np.all(np.abs(phi - g["snap_phi"]) <= PHI_RTOL * scale + 1e-15)
    np.testing.assert_allclose(w, g["restart_w"], rtol=1e-10, atol=1e-10)
    if int(g["counter"]) > 0:
        assert written == tuple(int(x) for x in g["restart_rng"])


def test_large_bulk_vs_oracle(srn, oracle_mod):
    """64x1x64 (the bulk workload's grid), 3 iterations, GPU vs oracle."""
    S = srn.configs.bulk2d(iters=3)
    w = srn.configs.uniform_fields(S.grid(), seed=5, amp=0.1)
    o = oracle_mod.Oracle(S)
    o.set_fields(w)
    o.set_iter(1)
    rec = o.iterate(3)
    r = runner_mod().Run(S, w, 1, (1, 2, 3))
    recs = r.step(3, keep_snapshots=False)
    for a, b in zip(recs, rec):
        assert abs(a.free_energy - b[1]) <= F_RTOL * abs(b[1])
    phi, _ = r.solver.get_densities()
    ophi, _ = o.densities()
    np.testing.assert_allclose(phi, ophi, rtol=PHI_RTOL, atol=1e-14)


def test_film_full_grid_vs_oracle(srn, oracle_mod):
    """192x1x96 thin film (the droplet workload's grid), 1 iteration, GPU vs oracle."""
    S = srn.configs.film2d(iters=1)
    w = srn.configs.droplet_fields(S, seed=9)
    m = srn.configs.substrate_mask(S)
    o = oracle_mod.Oracle(S)
    o.set_fields(w)
    o.set_masks(m)
    o.set_iter(1)
    rec = o.iterate(1)
    r = runner_mod().Run(S, w, 1, (1, 2, 3), m)
    out = r.step(1, keep_snapshots=False)[0]
    assert abs(out.free_energy - rec[0, 1]) <= F_RTOL * abs(rec[0, 1])
    np.testing.assert_allclose(out.q, rec[0, 21:38], rtol=1e-11)
    phi, _ = r.solver.get_densities()
    ophi, _ = o.densities()
    scale = np.maximum(np.abs(ophi).max(axis=1, keepdims=True), 1e-300)
    assert np.all(np.abs(phi - ophi) <= PHI_RTOL * scale + 1e-15)


def test_homogeneous_state_known_answer(srn):
    """w = 0, bulk melt: Q = 1, mu = 0 and F = chi_AB N phi_A phi_B with the
    discrete block fractions phi_A = (NS_X-1)/(NS_DBK-1), phi_B = NS_Y/(NS_DBK-1)
    (48/98 and 50/98 for NS = 100), every iteration."""
    S = srn.configs.bulk2d(iters=3)
    d = srn.derive(S)
    nsd, nsx, nsy = int(d.ns_dbk[0]), int(d.ns_dbk_x[0]), int(d.ns_dbk_y[0])
    expect = 20.0 * ((nsx - 1) / (nsd - 1)) * (nsy / (nsd - 1))
    w = np.zeros((14, 64 * 64))
    r = runner_mod().Run(S, w, 1, (1, 2, 3))
    recs = r.step(3, keep_snapshots=False)
    # Q = 1 in the first iteration; afterwards the update shifts w uniformly
    # (the block fractions differ from phi_avg), which moves Q but not F
    assert abs(recs[0].q[0] - 1.0) < 1e-13
    for rec in recs:
        assert abs(rec.free_energy - expect) < 1e-12
        assert rec.rms < 1e-13


def test_blend3d_full_grid_invariants(srn):
    """64^3 blend (the 3D workload's grid): each species' volume fraction is exact
    after normalisation by Q (mean_r of its blocks sums to VOL), F is finite and
    p has zero mean. (Single blocks of a diblock hold (NS_X-1)/(NS-1) of it, not f.)"""
    S = srn.configs.blend3d(iters=2)
    S.RELAXATION = 0
    w = srn.configs.uniform_fields(S.grid(), seed=11, amp=0.2, fields=tuple(range(9)))
    r = runner_mod().Run(S, w, 1, (1, 2, 3))
    rec = r.step(1, keep_snapshots=False)[0]
    assert np.isfinite(rec.free_energy)
    phi, tot = r.solver.get_densities()
    d = r.solver.derived[0]
    mean = phi.mean(axis=1)
    # A = dbk1-X + homo A, B = dbk1-Y + homo B, C = homo C, D+E = dbk2, F+G = dbk3, H+I = dbk4
    np.testing.assert_allclose(mean[0] + mean[1], 0.2 + 0.1 + 0.05, rtol=1e-12)
    np.testing.assert_allclose(mean[2], 0.05, rtol=1e-12)
    for a in (3, 5, 7):
        np.testing.assert_allclose(mean[a] + mean[a + 1], 0.2, rtol=1e-12)
    wout = r.solver.get_fields()
    assert abs(wout[13].mean()) < 1e-12


def test_batch_instances_match_solo_runs(srn):
    """Several chi points in one context give bit-identical results to solo contexts."""
    surfaces = [srn.configs.film2d(nx=32, nz=16, ns=64, chi_ab=a, iters=2) for a in (12.0, 20.0, 28.0)]
    w = srn.configs.droplet_fields(surfaces[0], seed=3, radius=1.2)
    m = srn.configs.substrate_mask(surfaces[0])
    with srn.Solver(surfaces, precision="fp64") as sv:
        for b in range(3):
            sv.set_fields(w, b)
            sv.set_masks(m, b)
            sv.set_iteration(1, b)
        outs = sv.iterate(2)
        batch_phi = [sv.get_densities(b)[0] for b in range(3)]
    for b, s in enumerate(surfaces):
        with srn.Solver(s, precision="fp64") as solo:
            solo.set_fields(w)
            solo.set_masks(m)
            solo.set_iteration(1)
            o = solo.iterate(2)
            assert o[-1][0].free_energy == outs[-1][b].free_energy
            np.testing.assert_array_equal(solo.get_densities()[0], batch_phi[b])


def test_graph_replay_matches_eager(srn, golden):
    g = golden("film2d")
    a = run_gpu(srn, g, use_graph=False)
    b = run_gpu(srn, g, use_graph=True)
    for x, y in zip(a.records, b.records):
        assert x.free_energy == y.free_energy


@pytest.mark.parametrize("case", ["bulk2d", "film2d", "blend3d"])
def test_fp32_form_error_bounds(case, srn, golden):
    """Precision form: FP32 propagators, FP64 reductions, on the golden runs'
    random (unconverged, grid-scale) starts: free energy within 3e-6 relative of
    the reference. Away from a saddle point F moves at first order with the FP32
    rounding of the densities; the 1e-6 contract is checked on converged states
    in test_gpu_precision.py."""
    g = golden(case)
    r = run_gpu(srn, g, precision="fp32")
    by_iter = {rec.iter: rec for rec in r.records}
    for row in g["free_energy"]:
        rec = by_iter[int(row[0])]
        assert abs(rec.free_energy - row[1]) <= 3e-6 * max(1.0, abs(row[1])), (case, rec.free_energy, row[1])


def test_film3d_mask_vs_oracle(srn, oracle_mod):
    """A 3D thin film (MASK 1: Dirichlet z, brush on the k = 0 plane), 16x10x12,
    two iterations of the plain form against the oracle."""
    S = srn.configs.film2d(nx=16, nz=12, ns=30, iters=2)
    S.LY = 10 * 0.125  # (LY = 1.0 would collapse the axis to one point, SCFT.c:103-105)
    nx, ny, nz = S.grid()
    assert (nx, ny, nz) == (16, 10, 12)
    i, j, k = srn.configs.idx_coords(nx, ny, nz)
    rng = np.random.default_rng(11)
    w = np.zeros((14, nx * ny * nz))
    for f in (0, 1, 2, 10):
        w[f] = rng.uniform(-0.5, 0.5, nx * ny * nz) + (2.0 if f < 2 else 0.0) * np.cos(2 * np.pi * i / nx)
    m = srn.configs.substrate_mask(S)
    o = oracle_mod.Oracle(S)
    o.set_fields(w)
    o.set_masks(m)
    o.set_iter(1)
    rec = o.iterate(2)
    with srn.Solver(S, precision="fp64") as sv:
        sv.set_fields(w)
        sv.set_masks(m)
        sv.set_iteration(1)
        out = sv.iterate(2)
        phi, _ = sv.get_densities()
    for k2 in range(2):
        assert abs(out[k2][0].free_energy - rec[k2, 1]) <= F_RTOL * abs(rec[k2, 1])
    ophi, _ = o.densities()
    scale = np.maximum(np.abs(ophi).max(axis=1, keepdims=True), 1e-300)
    assert np.all(np.abs(phi - ophi) <= PHI_RTOL * scale + 1e-15)
    o.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_density_unit_matches_funDensity(srn, precision):
    """scft_density (the kernel the iteration uses) against the reference's
    funMultiplyQs + funDensity on the same propagators (kat_density_2d)."""
    from conftest import load_golden
    g = load_golden("kat_density_2d")
    nx, ny, nz = (int(v) for v in g["grid"])
    S = srn.configs.bulk2d(nx=nx, nz=nz, iters=1)
    tol = 1e-13 if precision == "fp64" else 2e-7
    with srn.Solver(S, precision=precision) as sv:
        for (start, stop), phi in zip(g["blocks"], g["phi"]):
            got = sv.density(g["qf"], g["qb"], int(start), int(stop), float(g["Q"]))
            np.testing.assert_allclose(got, phi, rtol=tol, atol=0)


def _full_start(srn, name, S):
    """The start fields and grafting mask each full-size series was generated from."""
    if name == "blend3d_full":
        return srn.configs.uniform_fields(S.grid(), seed=1000, amp=0.1, fields=tuple(range(9))), None
    if name == "film2d_full":
        return srn.configs.droplet_fields(S, seed=1000), srn.configs.substrate_mask(S)
    return srn.configs.uniform_fields(S.grid(), seed=1000, amp=0.1, fields=(0, 1)), None


@pytest.mark.parametrize("name", ["bulk2d_full", "film2d_full", "blend3d_full"])
def test_full_size_configurations_match_reference(srn, name):
    """Each configuration at its full size against the reference's own first
    iterations from a seeded start: the 2D bulk melt (64x1x64, NS 100), the
    thin-film droplet (192x1x96, NS 128, MASK 1, brush) and the four-diblock
    blend (64^3, NS 128, 11 chains, noise from the drand48 replay): free energy,
    chemical potentials and RMS of every iteration."""
    g = load_golden(name)
    S = surface_from_json(srn, g["surface"])
    w0, mask3 = _full_start(srn, name, S)
    # the start must be the reference's: the generator's stream is checked, not trusted
    np.testing.assert_allclose(w0.sum(axis=1), g["w_sum"], rtol=0, atol=1e-9)
    np.testing.assert_allclose((w0 * w0).sum(axis=1), g["w_sumsq"], rtol=1e-14, atol=0)
    r = runner_mod().Run(S, w0, int(g["counter"]), tuple(int(x) for x in g["seed0"]), mask3, precision="fp64",
                         noise="device")
    r.run_to_end()
    by_iter = {rec.iter: rec for rec in r.records}
    assert len(g["free_energy"]) >= 6
    for row in g["free_energy"]:
        rec = by_iter[int(row[0])]
        assert abs(rec.free_energy - row[1]) <= F_RTOL * abs(row[1]), (row[0], rec.free_energy, row[1])
    for row in g["energies"]:
        np.testing.assert_allclose(by_iter[int(row[0])].mu, row[1:], rtol=1e-10, atol=1e-11)
    for row in g["deviations"]:
        rec = by_iter[int(row[0])]
        assert abs(rec.rms - row[1]) <= 1e-8 * abs(row[1]), (row[0], rec.rms, row[1])


@pytest.mark.parametrize("name", ["bulk2d_full", "film2d_full", "blend3d_full"])
def test_full_size_precision_form_error(srn, name):
    """The precision form (FP32 propagators, FP64 densities/Q/free energy/update)
    on the same full-size series: its free energy stays within 3e-6 relative of
    the reference's at every iteration."""
    g = load_golden(name)
    S = surface_from_json(srn, g["surface"])
    w0, mask3 = _full_start(srn, name, S)
    r = runner_mod().Run(S, w0, int(g["counter"]), tuple(int(x) for x in g["seed0"]), mask3, precision="fp32",
                         noise="device")
    r.run_to_end()
    by_iter = {rec.iter: rec for rec in r.records}
    rel = [abs(by_iter[int(row[0])].free_energy - row[1]) / abs(row[1]) for row in g["free_energy"]]
    print(name, "FP32 relative F error per iteration", ["%.1e" % x for x in rel])
    assert max(rel) <= 3e-6, rel
