"""The reference's main loop (SCFT.c:1088-1664) around the GPU library.

``Run`` owns a :class:`Solver` for one instance and reproduces what main()
does between and around iterations: the counter semantics (iterations
counter+1 .. ITER+1), the drand48 noise stream (drawn every iteration, even
when MF = 0), energies every D_WRT_ENERGIES iterations, snapshots and restart
files every D_WRT iterations and at iteration 1 — including the reference's
restart_random.dat, which holds the RNG state of the previous snapshot (the
restart seed at the first one): SCFT.c:1653-1662 prints through the pointer
of its first seed48 call after the second call has overwritten it.
"""
from __future__ import annotations

import os
import time
from pathlib import Path
from typing import List, Optional

import numpy as np

from . import solver as S
from .surface import Surface


class Run:
    def __init__(self, surface: Surface, w14: Optional[np.ndarray] = None, counter: int = 1, seed=(0, 0, 0),
                 mask3: Optional[np.ndarray] = None, precision: str = "fp64", outdir=None, use_graph: bool = False,
                 solver: Optional[S.Solver] = None, noise: str = "host"):
        self.surface = surface
        self.solver = solver or S.Solver(surface, precision=precision, use_graph=use_graph, noise=noise)
        self.device_noise = self.solver.noise_mode == "device"
        self.d = self.solver.derived[0]
        M = self.solver.M
        if counter == 0:
            # fresh start: zero fields (SCFT.c:799-842); the reference seeds drand48
            # from the clock, so a caller that wants a reproducible stream passes seed
            w14 = np.zeros((14, M))
        if w14 is None:
            raise ValueError("w14 is required for a restart (counter > 0)")
        self.solver.set_fields(w14)
        if surface.MASK:
            self.solver.set_masks(mask3 if mask3 is not None else np.zeros((3, M)))
        self.solver.set_iteration(counter)
        self.iter = int(counter)
        self.rng = tuple(int(x) for x in seed)
        if self.device_noise:
            self.solver.set_rng(self.rng)
        self.rng_saved = self.rng
        self.outdir = Path(outdir) if outdir is not None else None
        self.records: List[S.IterOut] = []
        self.snapshots = {}
        self.noise_ms = 0.0

    @property
    def n_remaining(self) -> int:
        return int(self.surface.ITER) - self.iter + 1

    def _mf(self, it: int) -> float:
        return 0.0 if it > int(self.surface.RELAXATION) else 1.0

    def step(self, n: int = 1, keep_snapshots: bool = True) -> List[S.IterOut]:
        """Run n iterations with the reference's side effects."""
        out = []
        s = self.surface
        for _ in range(n):
            it = self.iter + 1
            if self.device_noise:
                rec = self.solver.iterate(1)[0][0]
            else:
                t0 = time.perf_counter()
                need = self._mf(it) * s.DT_NOISE != 0.0
                noise, self.rng = S.noise_fill(self.rng, self.d, out=need)
                self.noise_ms += (time.perf_counter() - t0) * 1e3
                rec = self.solver.iterate(1, noise[None] if need else None)[0][0]
            self.iter = it
            out.append(rec)
            self.records.append(rec)
            if self.outdir is not None and it % int(s.D_WRT_ENERGIES) == 0:
                S.write_energies(self.outdir, self.d, rec)
            if it % int(s.D_WRT) == 0 or it == 1:
                if self.device_noise:
                    self.rng = self.solver.get_rng()
                written = self.rng_saved
                self.rng_saved = self.rng
                if self.outdir is not None or keep_snapshots:
                    phi, _ = self.solver.get_densities()
                    w = self.solver.get_fields()
                    if keep_snapshots:
                        self.snapshots[it] = (phi, w, written)
                    if self.outdir is not None:
                        S.write_snapshot(self.outdir, self.d, it, phi, w, written)
        return out

    def run_to_end(self, keep_snapshots: bool = False) -> List[S.IterOut]:
        return self.step(self.n_remaining, keep_snapshots=keep_snapshots)


def run_directory(path, precision: str = "fp64", use_graph: bool = False) -> Run:
    """Drop-in run in a directory laid out like the reference's working directory:
    parameters.h, counter.dat, restart_fields.dat / restart_random.dat (counter > 0),
    wMask.dat (MASK 1). Writes the same output files there."""
    path = Path(path)
    surface = Surface.from_parameters_h((path / "parameters.h").read_text())
    S.set_file_names(surface)
    try:
        d = S.derive(surface)
        if d.status != 0:
            S.write_volume_error(path, d.c.volume_sum)
            raise SystemExit(0)
        counter = S.read_counter(path)
        mask3 = S.read_mask(path, d) if surface.MASK else None
        if counter > 0:
            w14 = S.read_restart_fields(path, d)
            seed = S.read_restart_random(path)
        else:
            w14 = None
            ns = time.time_ns() % 1_000_000_000
            seed = (ns & 0xFFFF, (ns + 1) & 0xFFFF, (ns + 2) & 0xFFFF)
        S.write_run_params(path, surface, d, counter)
        r = Run(surface, w14, counter, seed, mask3, precision=precision, outdir=path, use_graph=use_graph)
        r.run_to_end()
    finally:
        S.set_file_names(None)
    return r


if __name__ == "__main__":
    import sys
    run_directory(sys.argv[1] if len(sys.argv) > 1 else os.getcwd())
