"""Iterative phase-diagram construction (the ICA workflow, README.md:59-127)
as a client of the serving loop.

The diagram is an n x n (chi_AB N, chi_AC N) grid repeated over three planes.
Each point is one SCFT solve. The first pass solves every point from a
synthetic seed; each later pass lets every point try the converged fields of
its neighbours (four in-plane, two across the cyclic plane order
P0 -> P1 -> P2 -> P0) not yet tried there, and keeps a trial when its free
energy is lower. A neighbour counts as tried for its current state: once a
neighbour's own state is replaced, its new field is tried again (marking the
neighbour alone would end the search after one pass, before a structure that
wins at one point can spread further). Passes repeat until one replaces
nothing. Every point keeps a
record with its current free energy, where its field came from and the
history of replaced states; with an output directory each record is written as
one JSON file per point.

Trials of one pass are submitted together and solved concurrently by the
server, so within a pass every trial uses its neighbour's state from the start
of the pass (the reference's pseudocode walks the points one after another;
the set of trials and the replacement rule are the same).
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from pathlib import Path
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from .serve import Completion, Request, Server
from .surface import Surface

Point = Tuple[int, int, int]  # (plane, i, j)


@dataclass
class PointState:
    free_energy: float
    source: str                      # "initial" or "P<plane>_<i>_<j>" of the seed's point
    converged: bool
    iterations: int
    fields: Optional[np.ndarray] = None
    tried: List[str] = field(default_factory=list)   # "<neighbour>@<its version>"
    history: List[dict] = field(default_factory=list)
    version: int = 0                                  # replacements so far


def point_name(p: Point) -> str:
    return f"P{p[0]}_{p[1]}_{p[2]}"


def neighbours(p: Point, n: int, planes: int = 3) -> List[Point]:
    plane, i, j = p
    out = []
    for di, dj in ((-1, 0), (1, 0), (0, -1), (0, 1)):
        if 0 <= i + di < n and 0 <= j + dj < n:
            out.append((plane, i + di, j + dj))
    if planes > 1:
        out.append(((plane + 1) % planes, i, j))
        out.append(((plane - 1) % planes, i, j))
    return list(dict.fromkeys(q for q in out if q != p))


class PhaseDiagram:
    """surface_fn(point) -> Surface; seed_fn(point) -> (w14, mask3 or None)."""

    def __init__(self, server: Server, cls: str, precision: str, n: int, surface_fn: Callable[[Point], Surface],
                 seed_fn: Callable[[Point], Tuple[np.ndarray, Optional[np.ndarray]]], planes: int = 3,
                 outdir=None):
        self.server, self.cls, self.precision = server, cls, precision
        self.n, self.planes = n, planes
        self.surface_fn, self.seed_fn = surface_fn, seed_fn
        self.outdir = Path(outdir) if outdir is not None else None
        self.points: List[Point] = [(p, i, j) for p in range(planes) for i in range(n) for j in range(n)]
        self.state: Dict[Point, PointState] = {}
        self.masks: Dict[Point, Optional[np.ndarray]] = {}
        self.trials: List[Tuple[Point, str, float, bool]] = []  # (point, source, F, converged)
        self.passes = 0
        self._rid = 0

    def _request(self, p: Point, w14: np.ndarray, key) -> Request:
        self._rid += 1
        return Request(rid=self._rid, cls=self.cls, surface=self.surface_fn(p), w14=w14, mask3=self.masks[p],
                       precision=self.precision, key=key, seed=(p[0] + 1, p[1] + 1, p[2] + 1))

    def _solve(self, reqs: Sequence[Request]) -> List[Completion]:
        keep = self.server.keep_fields
        self.server.keep_fields = True
        try:
            return self.server.run(reqs, realtime=False)
        finally:
            self.server.keep_fields = keep

    def first_pass(self) -> None:
        reqs = []
        for p in self.points:
            w, m = self.seed_fn(p)
            self.masks[p] = m
            reqs.append(self._request(p, w, (p, "initial")))
        for c in self._solve(reqs):
            p, src = c.key
            self.state[p] = PointState(c.free_energy, src, c.converged, c.iterations, c.fields)
            self.trials.append((p, src, c.free_energy, c.converged))
        self.passes = 1
        self._write()

    def update_pass(self) -> int:
        """One pass of neighbour trials; returns the number of replacements."""
        reqs = []
        for p in self.points:
            st = self.state[p]
            for q in neighbours(p, self.n, self.planes):
                name = point_name(q)
                mark = f"{name}@{self.state[q].version}"
                if mark in st.tried:
                    continue
                st.tried.append(mark)
                reqs.append(self._request(p, self.state[q].fields, (p, name)))
        if not reqs:
            return 0
        best: Dict[Point, Completion] = {}
        for c in self._solve(reqs):
            p, src = c.key
            self.trials.append((p, src, c.free_energy, c.converged))
            if not np.isfinite(c.free_energy):
                continue
            if p not in best or c.free_energy < best[p].free_energy:
                best[p] = c
        self.passes += 1
        replaced = 0
        for p, c in best.items():
            st = self.state[p]
            if c.free_energy < st.free_energy:
                st.history.append({"pass": self.passes - 1, "free_energy": st.free_energy, "source": st.source,
                                   "converged": st.converged, "iterations": st.iterations})
                st.free_energy, st.source, st.converged, st.iterations = (c.free_energy, c.key[1], c.converged,
                                                                          c.iterations)
                st.fields = c.fields
                st.version += 1
                replaced += 1
        self._write()
        return replaced

    def run(self, max_passes: int = 50) -> int:
        if not self.state:
            self.first_pass()
        while self.passes < max_passes:
            if self.update_pass() == 0:
                break
        return self.passes

    def record(self, p: Point) -> dict:
        st = self.state[p]
        return {"point": point_name(p), "plane": p[0], "i": p[1], "j": p[2], "free_energy": st.free_energy,
                "source": st.source, "converged": st.converged, "iterations": st.iterations, "version": st.version,
                "neighbours": [point_name(q) for q in neighbours(p, self.n, self.planes)], "tried": list(st.tried),
                "history": list(st.history)}

    def _write(self) -> None:
        if self.outdir is None:
            return
        self.outdir.mkdir(parents=True, exist_ok=True)
        for p in self.points:
            (self.outdir / f"{point_name(p)}.json").write_text(json.dumps(self.record(p), indent=1))

    def free_energies(self) -> np.ndarray:
        F = np.full((self.planes, self.n, self.n), np.nan)
        for (pl, i, j), st in self.state.items():
            F[pl, i, j] = st.free_energy
        return F
