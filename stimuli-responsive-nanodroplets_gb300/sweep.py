"""The 2D droplet sweep: n x n (chi_AB N, chi_AC N) points of the thin-film
droplet chemistry on uneven grids, each run until RMS(phi_tot - 1) < tol.

Each point is one instance of a :class:`Batch`; grid size and NS are drawn per
point from a seed (``configs.sweep_surfaces``), the start is a half-disk
droplet scaled to the box with seeded w noise, and S1 is grafted on the k = 0
layer. ``run_sweep`` returns per-instance results and the wall time, from
which solves/hour follows.
"""
from __future__ import annotations

import time
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import configs
from .batch import Batch, BatchResult
from .surface import Surface

SWEEP_SIZES = ((64, 64), (96, 64), (128, 96), (192, 96), (192, 128))


def droplet_radius(s: Surface) -> float:
    """6 R_g on the 24 x 12 film; smaller boxes get a droplet that fits."""
    return float(min(6.0, 0.3 * s.LX, 0.6 * s.LZ))


def sweep_inputs(surfaces: Sequence[Surface], seed: int = 100):
    """(w14, mask3) per instance: seeded droplet start and the substrate mask."""
    out = []
    for i, s in enumerate(surfaces):
        w = configs.droplet_fields(s, seed=seed + i, radius=droplet_radius(s))
        out.append((w, configs.substrate_mask(s)))
    return out


@dataclass
class SweepRun:
    results: List[BatchResult]
    wall_s: float
    groups: int
    precision: str

    @property
    def converged(self) -> int:
        return sum(r.converged for r in self.results)

    @property
    def solves_per_hour(self) -> float:
        return self.converged * 3600.0 / self.wall_s if self.wall_s > 0 else 0.0

    @property
    def instance_iterations(self) -> int:
        return sum(r.iterations for r in self.results)


def make_batch(surfaces, inputs, precision="fp32", rms_tol=1e-6, use_graph=True) -> Batch:
    b = Batch(surfaces, precision=precision, use_graph=use_graph, noise="device")
    for i, (w, m) in enumerate(inputs):
        b.set_fields(i, w)
        b.set_masks(i, m)
        b.set_iteration(i, 1)
        b.set_rng(i, (11 + i, 22, 33))
        b.set_stop(i, rms_tol)
    return b


def run_sweep(n: int = 16, precision: str = "fp32", rms_tol: float = 1e-6, max_iter: int = 20000, chunk: int = 200,
              seed: int = 3, sizes=SWEEP_SIZES, ns_range=(64, 128), surfaces: Optional[Sequence[Surface]] = None,
              use_graph: bool = True) -> SweepRun:
    if surfaces is None:
        surfaces = configs.sweep_surfaces(n, seed=seed, sizes=sizes, ns_range=ns_range)
        for s in surfaces:
            s.ITER = max_iter + 1
            s.D_WRT = s.ITER
    inputs = sweep_inputs(surfaces)
    with make_batch(surfaces, inputs, precision, rms_tol, use_graph) as b:
        t0 = time.perf_counter()
        res = b.run(max_iter, chunk)
        wall = time.perf_counter() - t0
        groups = b.groups
    return SweepRun(res, wall, groups, precision)


def summary(run: SweepRun) -> dict:
    it = np.array([r.iterations for r in run.results])
    return {"precision": run.precision, "instances": len(run.results), "converged": run.converged,
            "groups": run.groups, "wall_s": run.wall_s, "solves_per_hour": run.solves_per_hour,
            "iters_median": float(np.median(it)), "iters_max": int(it.max()),
            "instance_iters_per_s": run.instance_iterations / run.wall_s if run.wall_s > 0 else 0.0}
