"""FP32x2 form (propagators in double-float arithmetic on FP32 pairs, FP64
reductions) against the reference's own outputs (tests/golden) and the plain
FP64 form.

Double-float values carry ~48 significant bits (rounding 2^-48 against FP64's
2^-53). Measured on GB300 the form stays within ~1e-14 of the reference's
FFTW-double outputs (propagator slices, densities, free energies), inside the
plain form's own contract (1e-10 densities, 1e-9 free energy); it is held here
to 1e-12 on all three. It is the finishing form below the FP32 form's RMS
floor, where it must reach the FP64 fixed point: a relaxed film state within
1e-10 of the plain form's free energy (RMS to 1e-8).
"""
import importlib

import numpy as np
import pytest

from conftest import load_golden, surface_from_json

pytestmark = pytest.mark.gpu

CASES = ["bulk2d", "film2d", "blend3d", "quirks", "seed"]


@pytest.mark.parametrize("tag", ["periodic2d", "dirichlet2d", "periodic3d"])
def test_propagate_matches_funPDESolver(tag, srn):
    g = load_golden(f"kat_prop_{tag}")
    S = surface_from_json(srn, g["surface"])
    with srn.Solver(S, precision="fp32x2") as sv:
        q = sv.propagate(g["q0"], g["w"], g["q"].shape[0] - 1)
    scale = np.abs(g["q"]).max()
    err = np.abs(q - g["q"]).max() / scale
    print(tag, "max error / max |q|", err)
    np.testing.assert_allclose(q, g["q"], rtol=1e-12, atol=1e-13 * scale)


@pytest.mark.parametrize("case", CASES)
def test_iterations_match_reference(case, srn, golden):
    g = golden(case)
    S = g["S"]
    counter = int(g["counter"])
    runner = importlib.import_module("stimuli-responsive-nanodroplets_gb300.runner")
    r = runner.Run(S, g["w0"] if counter > 0 else None, counter, tuple(int(x) for x in g["seed0"]), g["mask3"],
                   precision="fp32x2")
    r.run_to_end(keep_snapshots=True)
    by_iter = {rec.iter: rec for rec in r.records}
    worst = 0.0
    for row in g["free_energy"]:
        rec = by_iter[int(row[0])]
        rel = abs(rec.free_energy - row[1]) / max(1.0, abs(row[1]))
        worst = max(worst, rel)
        assert rel <= 1e-12, (case, row[0], rec.free_energy, row[1])
    for row in g["deviations"]:
        rec = by_iter[int(row[0])]
        assert abs(rec.rms - row[1]) <= 1e-10 * abs(row[1]) + 1e-13
    phi, w, written = r.snapshots[int(g["snap_iter"])]
    scale = np.maximum(np.abs(g["snap_phi"]).max(axis=1, keepdims=True), 1e-300)
    print(case, "F rel", worst, "phi", float((np.abs(phi - g["snap_phi"]) / scale).max()))
    assert np.all(np.abs(phi - g["snap_phi"]) <= 1e-12 * scale + 1e-15)


def test_relaxed_film_matches_plain_form(srn):
    """A 64x32 thin film (MASK 1: dense z pass, FFT x pass) relaxed 400
    iterations from a droplet seed in both forms: the same free energy and RMS
    trajectory (free energy to 1e-10, RMS to 1e-8: 400 iterations of the
    update carry the forms' 1e-14 differences), with the FP32x2 form on the
    per-axis passes."""
    cfg = srn.configs
    S = cfg.film_point(20.0, 40.0, cfg.PLANES[0], nx=64, nz=32, ns=64)
    w0 = cfg.droplet_fields(S, seed=2)
    m = cfg.substrate_mask(S)
    out = {}
    for prec in ("fp64", "fp32x2"):
        with srn.Solver([S], precision=prec) as sv:
            sv.set_fields(w0, 0)
            sv.set_masks(m, 0)
            sv.set_iteration(1, 0)
            out[prec] = [o[0] for o in sv.iterate(400)]
            if prec == "fp32x2":
                assert sv.timing().get("fused_chain", 0) == 0
    for a, b in zip(out["fp64"], out["fp32x2"]):
        assert abs(a.free_energy - b.free_energy) <= 1e-10 * abs(a.free_energy)
        assert abs(a.rms - b.rms) <= 1e-8 * a.rms + 1e-14
