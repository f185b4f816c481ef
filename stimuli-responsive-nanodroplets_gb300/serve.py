"""Serving loop: continuous batching of phase-diagram solve requests.

Requests (a chi point, a plane and a seed field) arrive over time. The server
keeps one context per (shape class, precision) with a fixed number of slots;
the slot counts come from a device-memory budget (every slot's fields,
propagators and densities are allocated once and stay resident in HBM), so a
request is admitted when a slot of its class is free. Each round enqueues a
chunk of iterations on every context with busy slots (the contexts' streams
run side by side), then collects the records: a slot whose instance met the
RMS tolerance, or ran out of iterations, completes its request and takes the
next queued one at once (scft_set_surface + scft_set_fields on the freed
slot; idle slots are frozen and cost nothing on the device). Every pool runs
its own rounds: the loop polls the pools without blocking, collects a pool as
soon as its chunk has finished and refills and relaunches it at once, so a
pool of fast 2D solves is never held back by a pool of slower 3D ones.

Per-instance arithmetic does not depend on the other slots (reductions run in
a fixed order per instance, operator tables depend only on the instance's own
parameters), so a request's result is the same alone and in the mix.

The reference has no serving layer (one process per solve, SCFT.c:1088); the
request stream stands in for the phase-diagram workflow of README.md:59-127.
"""
from __future__ import annotations

import collections
import dataclasses
import time
from dataclasses import dataclass
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from .solver import Solver, device_memory
from .surface import Surface


@dataclass
class Request:
    rid: int
    cls: str                     # shape class, e.g. "film2d" or "bulk3d"
    surface: Surface
    w14: np.ndarray
    mask3: Optional[np.ndarray] = None
    precision: str = "fp32"
    arrival: float = 0.0         # seconds after the start of the stream
    key: tuple = ()              # caller's label, e.g. (plane, i, j, trial)
    seed: Tuple[int, int, int] = (11, 22, 33)


@dataclass
class Completion:
    rid: int
    key: tuple
    cls: str
    precision: str
    arrival: float
    admitted: float
    finished: float
    iterations: int
    free_energy: float
    rms: float
    converged: bool
    status: int
    fields: Optional[np.ndarray] = None

    @property
    def latency(self) -> float:
        """Time to converged: arrival to completion, queueing included."""
        return self.finished - self.arrival


class Pool:
    """One context of `slots` instances of one shape class and precision.

    template: a surface with the class's grid and composition and the largest
    NS the pool serves (it fixes the contour slices allocated per slot)."""

    def __init__(self, cls: str, template: Surface, slots: int, precision: str, use_graph: bool = True,
                 solver=None, chunk: Optional[int] = None):
        self.cls, self.precision, self.slots = cls, precision, int(slots)
        self.chunk = chunk  # iterations per round (None: the server's)
        # pools run side by side: launch forms tuned on one pool alone would not be the
        # fastest with the others in flight, so pools keep the heuristic forms
        self.sv = solver if solver is not None else Solver([template] * self.slots, precision=precision,
                                                            use_graph=use_graph, noise="device", autotune=False)
        zero = np.zeros((14, self.sv.M))
        for b in range(self.slots):
            self.sv.set_fields(zero, b)
            self.sv.set_iteration(1, b)
            self.sv.freeze(b)
        self.free: List[int] = list(range(self.slots))[::-1]
        self.busy: Dict[int, Tuple[Request, float, int]] = {}
        self.in_flight = 0

    @property
    def device_bytes(self) -> int:
        return self.sv.device_bytes

    def admit(self, req: Request, now: float, rms_tol: float) -> None:
        b = self.free.pop()
        sv = self.sv
        sv.set_surface(b, req.surface)
        sv.set_fields(req.w14, b)
        if req.mask3 is not None:
            sv.set_masks(req.mask3, b)
        sv.set_rng(req.seed, b)
        sv.set_stop(rms_tol, b)
        sv.set_iteration(1, b)
        self.busy[b] = (req, now, 0)

    def launch(self, chunk: int) -> bool:
        if not self.busy or self.in_flight:
            return False
        n = self.chunk or chunk
        self.sv.iterate_async(n)
        self.in_flight = n
        return True

    def ready(self) -> bool:
        return bool(self.in_flight) and self.sv.iterate_ready()

    def collect(self, now_fn: Callable[[], float], max_iter: int, keep_fields: bool) -> List[Completion]:
        if not self.in_flight:
            return []
        recs = self.sv.iterate_wait(allow_nonfinite=True)  # a failed slot ends its own request only
        now = now_fn()
        self.in_flight = 0
        done = []
        for b, (req, t_adm, ran) in list(self.busy.items()):
            last = recs[-1][b]
            ran_now = int(last.iter) - 1  # admitted at iIter 1
            if last.converged or ran_now >= max_iter or last.status != 0:
                fields = self.sv.get_fields(b) if keep_fields else None
                done.append(Completion(req.rid, req.key, self.cls, self.precision, req.arrival, t_adm, now,
                                       int(ran_now), last.free_energy, last.rms, bool(last.converged), last.status,
                                       fields))
                self.sv.freeze(b)
                del self.busy[b]
                self.free.append(b)
            else:
                self.busy[b] = (req, t_adm, ran_now)
        return done


class BudgetError(ValueError):
    """The memory budget does not hold one slot of the class."""


def slots_for_budget(template: Surface, precision: str, budget_bytes: int, max_slots: int = 512,
                     device: int = 0, reserve_frac: float = 0.05) -> int:
    """Slots of one class that fit a device-memory budget (bytes per slot
    measured on a two-slot context, so shared tables are not counted twice).
    The budget is capped by the device's free memory less reserve_frac of its
    total; a budget that cannot hold one slot raises BudgetError instead of
    over-committing the device."""
    with Solver([template], precision=precision, noise="device", device=device) as one:
        b1 = one.device_bytes
    with Solver([template, template], precision=precision, noise="device", device=device) as two:
        b2 = two.device_bytes
    per_slot = max(1, b2 - b1)
    fixed = max(0, b1 - per_slot)
    free, total = device_memory(device)
    usable = min(int(budget_bytes), free - int(reserve_frac * total))
    n = (usable - fixed) // per_slot
    if n < 1:
        raise BudgetError(f"a budget of {budget_bytes} bytes ({usable} usable of {free} free) holds no slot of "
                          f"{fixed + per_slot} bytes")
    return int(min(max_slots, n))


class Server:
    """Continuous-batching scheduler over pools keyed by (class, precision)."""

    def __init__(self, pools: Dict[Tuple[str, str], Pool], rms_tol: float = 1e-6, max_iter: int = 20000,
                 chunk: int = 50, keep_fields: bool = False):
        self.pools = pools
        self.rms_tol, self.max_iter, self.chunk = rms_tol, max_iter, chunk
        self.keep_fields = keep_fields

    def run(self, requests: Sequence[Request], realtime: bool = True) -> List[Completion]:
        """Serve requests in arrival order. realtime: arrivals follow the wall
        clock (a request is visible only after its arrival time)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        for r in reqs:
            if (r.cls, r.precision) not in self.pools:
                raise KeyError(f"no pool for class {r.cls!r} at {r.precision}")
        if not realtime:
            reqs = [dataclasses.replace(r, arrival=0.0) for r in reqs]
        queues: Dict[Tuple[str, str], collections.deque] = {k: collections.deque() for k in self.pools}
        t0 = time.perf_counter()

        def now_fn() -> float:
            return time.perf_counter() - t0

        nxt = 0
        out: List[Completion] = []
        while nxt < len(reqs) or any(queues[k] for k in queues) or any(p.busy for p in self.pools.values()):
            progressed = False
            now = now_fn()
            while nxt < len(reqs) and reqs[nxt].arrival <= now:
                queues[(reqs[nxt].cls, reqs[nxt].precision)].append(reqs[nxt])
                nxt += 1
            for k, pool in self.pools.items():
                if pool.in_flight:
                    if not pool.ready():
                        continue
                    out.extend(pool.collect(now_fn, self.max_iter, self.keep_fields))
                    progressed = True
                while queues[k] and pool.free:
                    pool.admit(queues[k].popleft(), now_fn(), self.rms_tol)
                if pool.launch(self.chunk):
                    progressed = True
            if not progressed:
                busy = any(p.in_flight for p in self.pools.values())
                wait = 0.0005 if busy else (max(0.0, min(0.01, reqs[nxt].arrival - now_fn())) if nxt < len(reqs)
                                            else 0.0)
                time.sleep(wait)
        return out

    def close(self):
        for p in self.pools.values():
            p.sv.close()


def latency_stats(done: Sequence[Completion], wall_s: float) -> dict:
    lat = np.array([c.latency for c in done]) if done else np.zeros(1)
    conv = sum(c.converged for c in done)
    return {"requests": len(done), "converged": conv, "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "solves_per_hour": conv * 3600.0 / wall_s if wall_s > 0 else 0.0}
