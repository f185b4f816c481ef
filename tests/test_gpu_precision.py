"""Precision form (FP32 propagators, FP64 densities/Q/free energy/update) on
converged states: free energies within 1e-6 relative of the plain FP64 form and
the same lowest-F winner among competing structures.

Competing structures: lamellae with 1, 2 and 3 periods across the 64x64 bulk
melt (chi_AB N = 20, f = 0.5), all instances of one batch, relaxed from
sinusoidal fields in both forms.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ITERS = 1200


def lamellar_fields(srn, S, periods, amp=3.0):
    nx, ny, nz = S.grid()
    i, j, k = srn.configs.idx_coords(nx, ny, nz)
    w = np.zeros((14, nx * ny * nz))
    phase = np.cos(2.0 * np.pi * periods * i / nx)
    w[0] = amp * phase
    w[1] = -amp * phase
    return w


def relax(srn, precision, surfaces, fields):
    with srn.Solver(surfaces, precision=precision) as sv:
        for b, w in enumerate(fields):
            sv.set_fields(w, b)
            sv.set_iteration(1, b)
        out = sv.iterate(ITERS)
    return out[-1]


def test_converged_free_energies_and_winner(srn):
    S = srn.configs.bulk2d(iters=ITERS + 1)
    structures = (1, 2, 3)
    surfaces = [S.copy() for _ in structures]
    fields = [lamellar_fields(srn, S, p) for p in structures]
    f64 = relax(srn, "fp64", surfaces, fields)
    f32 = relax(srn, "fp32", surfaces, fields)
    F64 = np.array([r.free_energy for r in f64])
    F32 = np.array([r.free_energy for r in f32])
    rel = np.abs(F32 - F64) / np.abs(F64)
    print("F64", F64, "F32", F32, "rel", rel, "rms", [r.rms for r in f64])
    assert np.all(rel < 1e-6), rel
    assert int(np.argmin(F32)) == int(np.argmin(F64))
