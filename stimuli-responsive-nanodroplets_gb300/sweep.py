"""The 2D droplet sweep: n x n (chi_AB N, chi_AC N) points of the thin-film
droplet chemistry on uneven grids, each run until RMS(phi_tot - 1) < tol.

Each point is one instance of a :class:`Batch`; grid size and NS are drawn per
point from a seed (``configs.sweep_surfaces``), the start is a half-disk
droplet scaled to the box with seeded w noise, and S1 is grafted on the k = 0
layer. ``run_sweep`` returns per-instance results and the wall time, from
which solves/hour follows.
"""
from __future__ import annotations

import queue
import threading
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


#: Hand-over of the precision form to the plain FP64 form (run_finished): an
#: instance moves once its FP32 RMS is below SWITCH_RMS and has stopped falling
#: (less than STALL_GAIN over STALL_ROUND iterations), i.e. once it sits on the
#: FP32 form's RMS floor (3e-6 - 9e-6 on the sweep shapes: FP32 rounding of the
#: propagators puts that much relative noise into phi_tot), or once it is below
#: FLOOR_RMS, under which the FP32 form does not go.
SWITCH_RMS = 2e-5
FLOOR_RMS = 3e-6
STALL_ROUND = 400
STALL_GAIN = 0.8


@dataclass
class FinishedResult:
    iterations: int       # both phases
    iterations_fp32: int
    rms: float
    free_energy: float
    converged: bool       # RMS < rms_tol within max_iter iterations in all
    status: int


def run_finished(surfaces: Sequence[Surface], inputs, rms_tol: float, max_iter: int, switch_rms: float = SWITCH_RMS,
                 chunk: int = 200, use_graph: bool = True, stall_round: int = STALL_ROUND,
                 stall_gain: float = STALL_GAIN, floor_rms: float = FLOOR_RMS, finish: str = "fp32x2"):
    """The precision form run to an RMS below its FP32 floor: every instance
    iterates in FP32 until it sits on the FP32 floor (RMS < switch_rms and no
    longer falling by stall_gain per stall_round iterations, or RMS < floor_rms),
    then continues from its fields in the `finish` form until RMS < rms_tol:
    "fp32x2" (double-float propagators, ~48 significant bits, several times
    faster than FP64 on GB300) or "fp64" (the plain form). max_iter bounds each
    instance's two phases together. The iteration is the reference's update in
    both phases; only the propagators' precision changes at the hand-over.

    The two phases overlap: the finishing batch (every instance, each frozen
    until it is handed over) is driven by a second host thread, which arms
    instances between its rounds as the FP32 batch hands them over, so
    finishing starts while the FP32 batch still runs its slower instances.
    The two batches are separate contexts on their own streams. Returns
    (results, wall seconds, seconds of the FP32 phase), timed from the first
    iteration (batch creation excluded, as in the single-form runs)."""
    n = len(surfaces)
    used = [0] * n
    last_rms = [float("inf")] * n
    out: List[Optional[FinishedResult]] = [None] * n
    handq: "queue.Queue" = queue.Queue()
    errors: list = []
    abort = threading.Event()            # the FP32 loop failed: the finisher stops at its next round
    b = make_batch(surfaces, inputs, "fp32", rms_tol, use_graph)
    bf = None
    try:
        bf = Batch(surfaces, precision=finish, use_graph=use_graph, noise="device")
        for i, (w, m) in enumerate(inputs):
            bf.set_fields(i, w)          # placeholders until the hand-over brings the FP32 fields
            bf.set_masks(i, m)
            bf.freeze(i)

        def finisher():
            live = {}                    # instance -> FP32 iterations it ran
            ran = {}                     # instance -> iterations in the finishing form
            fp32_over = False
            try:
                while not abort.is_set():
                    pending = []
                    if not live and not fp32_over:
                        pending.append(handq.get())          # idle: wait for the next hand-over
                    while True:
                        try:
                            pending.append(handq.get_nowait())
                        except queue.Empty:
                            break
                    for item in pending:
                        if item is None:
                            fp32_over = True
                            continue
                        i, w, it_after, used32 = item
                        bf.set_fields(i, w)
                        bf.set_iteration(i, it_after)       # re-arms the frozen instance
                        bf.set_rng(i, (11 + i, 22, 33))
                        bf.set_stop(i, rms_tol)
                        live[i] = used32
                        ran[i] = 0
                    if not live:
                        if fp32_over:
                            return
                        continue
                    res = bf.run(chunk, chunk)
                    for i in list(live):
                        r = res[i]
                        ran[i] += r.iterations
                        total = live[i] + ran[i]
                        if r.converged or r.status != 0 or total >= max_iter:
                            # the result as the instance leaves; a capped one is frozen here,
                            # so its stop is never mistaken for convergence
                            out[i] = FinishedResult(total, live[i], r.rms, r.free_energy,
                                                    bool(r.converged) and total <= max_iter, r.status)
                            if not r.converged:
                                bf.freeze(i)
                            del live[i]
            except BaseException as e:                     # reported by the caller
                errors.append(e)

        t0 = time.perf_counter()
        th = threading.Thread(target=finisher, name="fp32-finish", daemon=True)
        th.start()
        try:
            active = set(range(n))
            while active:
                res = b.run(stall_round, chunk)
                for i in list(active):
                    r = res[i]
                    used[i] += r.iterations
                    done = r.converged or r.status != 0 or used[i] >= max_iter
                    if not done and r.rms < switch_rms and (r.rms > stall_gain * last_rms[i] or r.rms < floor_rms):
                        handq.put((i, b.get_fields(i), r.iter, used[i]))
                        b.freeze(i)
                        active.discard(i)
                    elif done:
                        out[i] = FinishedResult(used[i], used[i], r.rms, r.free_energy, bool(r.converged), r.status)
                        b.freeze(i)
                        active.discard(i)
                    last_rms[i] = r.rms
                if errors:
                    break
            t1 = time.perf_counter()
        except BaseException:
            abort.set()
            raise
        finally:
            handq.put(None)
            th.join()
        if errors:
            raise errors[0]
        return out, time.perf_counter() - t0, t1 - t0
    finally:
        b.close()
        if bf is not None:
            bf.close()


def summary(run: SweepRun) -> dict:
    it = np.array([r.iterations for r in run.results])
    return {"precision": run.precision, "instances": len(run.results), "converged": run.converged,
            "groups": run.groups, "wall_s": run.wall_s, "solves_per_hour": run.solves_per_hour,
            "iters_median": float(np.median(it)), "iters_max": int(it.max()),
            "instance_iters_per_s": run.instance_iterations / run.wall_s if run.wall_s > 0 else 0.0}
