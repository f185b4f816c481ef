"""Benchmark: SCFT iterations/s of the thin-film nanodroplet system on one GB300.

Workload (default): the droplet system of the 2D thin-film configuration
(MASK 1, grid 192x1x96, NS = 128: AB diblock f = 0.5 at VOL 0.20, homopolymer C
solvent, brush S1 at z = 0; 502 contour steps per iteration), as a phase-diagram
batch of B instances on a chi_AB N x chi_AC N sweep, each started from a seeded
half-disk droplet. A step is one SCFT iteration of every instance.

value     instance-iterations/s of the FP32-propagator / FP64-reduction form,
          inputs resident in HBM, CUDA events on the library's stream.
e2e       the same through the C ABI with host buffers: per step the restart
          fields of every instance go host->device (pinned), one iteration
          runs, fields and densities come back device->host.
fp64_plain  the plain FP64 form (the drop-in) on the same batch.
roofline  propagator passes: algorithmic bytes 3*P*M per contour step per
          chain (read q_s, read exp(-w ds/2), write q_{s+1}) over the time of the
          propagator launches.
cpu_baseline  the CPU restatement of SCFT.c (oracle/, same algorithm, data
          layout and FFT code as the reference built here) on the host cores,
          one instance per core, bounded sample.

--impl reference times that CPU implementation alone on the same workload.
Under torchrun every rank runs its own batch (replicas: SCFT solves are
independent, there is no collective on the data path).
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
PKG = "stimuli-responsive-nanodroplets_gb300"
PEAKS = ROOT / "MEASURED_PEAKS.json"
TRAFFIC = ROOT / "profiles" / "traffic.json"
METRIC = "SCFT iters/s & solves/hr, fused FP32 vs plain FP64 on 1 GB300; p50/p99 solve latency"


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(pg, values, device):
    """Element-wise maximum of per-rank timings (the slowest rank sets the job's
    time); pg is torch.distributed or None for one process."""
    if pg is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]


def job_rate(world: int, per_rank_units: int, ms: float) -> float:
    """Whole-job throughput: every rank processes per_rank_units per step (weak
    scaling, replicas), the step time is the maximum over ranks."""
    return world * per_rank_units / (ms * 1e-3)


def workload_surfaces(srn, name: str, batch: int):
    n = int(round(np.sqrt(batch)))
    out = []
    for b in range(batch):
        a, c = divmod(b, max(n, 1))
        chi_ab = 10.0 + 20.0 * (a % n) / max(n - 1, 1)
        chi_ac = 20.0 + 40.0 * c / max(n - 1, 1)
        if name == "film2d":
            out.append(srn.configs.film2d(chi_ab=chi_ab, chi_ac=chi_ac))
        elif name == "bulk2d":
            s = srn.configs.bulk2d()
            s.set_chi("A", "B", chi_ab)
            out.append(s)
        elif name == "blend3d":
            out.append(srn.configs.blend3d(seed=2 + b))
        elif name == "bulk3d":
            out.append(srn.configs.bulk3d_point(chi_ab, chi_ac, srn.configs.PLANES[b % 3], ns=100))
        else:
            raise SystemExit(f"unknown workload {name}")
    return out


def initial_fields(srn, s, seed):
    if s.MASK:
        return srn.configs.droplet_fields(s, seed=seed), srn.configs.substrate_mask(s)
    nf = 9 if s.VOL_DBK[1] > 0 else 2
    return srn.configs.uniform_fields(s.grid(), seed=seed, amp=0.1, fields=tuple(range(nf))), None


def start_iteration(s) -> int:
    """Restart counter of timed runs (the noise, where on, comes from the
    device replay of the drand48 stream)."""
    return 1


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.rows = []
        if self.proc is None:
            return
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for line in out.splitlines():
            v = [x.strip() for x in line.split(",")]
            if len(v) == 7:
                self.rows.append(v)

    def summary(self):
        rows = getattr(self, "rows", [])
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[3 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def algorithmic_bytes(solver, psize: int) -> float:
    """Sum over chains of (len-1) contour steps x 3*P*M, per instance-iteration."""
    d = solver.derived[0]
    steps = 0
    for k in range(4):
        if d.ns_dbk[k] > 0:
            steps += 2 * (int(d.ns_dbk[k]) - 1)
    for h in range(10):
        if d.ns_homo[h] > 0:
            steps += int(d.ns_homo[h]) - 1
    for k in range(3):
        if d.ns_s[k] > 0:
            steps += 2 * (int(d.ns_s[k]) - 1)
    return float(steps) * 3 * psize * solver.M, steps


def measure_form(srn, surfaces, precision: str, steps: int, warmup: int, device: int, sync, e2e_steps: int,
                 e2e_parts: int = 8):
    B = len(surfaces)
    sv = srn.Solver(surfaces, precision=precision, device=device, noise="device")
    init = [initial_fields(srn, s, 1000 + b) for b, s in enumerate(surfaces)]
    for b, (w, m) in enumerate(init):
        sv.set_fields(w, b)
        if m is not None:
            sv.set_masks(m, b)
        sv.set_iteration(start_iteration(surfaces[b]), b)
        sv.set_rng((11 + b, 22, 33), b)
    sv.iterate(warmup)
    sv.enable_timing(True)
    sync()
    with ClockSampler(device) as clk:
        t0 = time.perf_counter()
        outs = sv.iterate(steps)
        wall = time.perf_counter() - t0  # the sampler's start and stop stay outside
    t = sv.timing()
    sync()
    bytes_iter, steps_iter = algorithmic_bytes(sv, 8 if precision == "fp64" else 4)
    ms = t["total_ms"]
    res = {
        "value": B * steps / (ms * 1e-3),
        "ms_per_step": ms / steps,
        "wall_ms_per_step": wall * 1e3 / steps,
        "prop_ms_per_step": t["prop_ms"] / steps,
        "prop_launches_per_step": t["prop_launches"] / steps,
        "gpu_launches": int(t["kernel_launches"]),
        "clocks": clk.summary(),
        "free_energy_first_instance": outs[-1][0].free_energy,
        "algorithmic_bytes_per_step": bytes_iter * B,
        "contour_steps_per_instance_iteration": steps_iter,
        "device_bytes": sv.device_bytes,
        "threads_per_line": int(t["threads_per_line"]),
        "kernel": {1: f"k_chain2d<float,{sv.grid[0]},{sv.grid[2]}> (persistent fused contour loop)",
                   2: "k_chain3d (64^3 contour loop, one 8-CTA cluster per chain)"}.get(
                       t["fused_chain"], "k_pass_fft + k_pass_dense (per-axis passes)"),
    }
    res["achieved_gbs"] = bytes_iter * B / (t["prop_ms"] * 1e-3 / steps) / 1e9
    # end to end through the C ABI with pinned host buffers: per step the restart
    # fields of every instance go in, one iteration runs, fields and densities
    # come back. Every step restarts from the same fields (the state after the
    # timed steps above), so the measured iterations stay in the regime the
    # device-resident number was taken in, also for a workload that diverges a
    # few iterations later. The batch is split into `e2e_parts` contexts on their
    # own streams and software-pipelined: a part's transfers of step k overlap the
    # other parts' iterations (each part still waits for its own outputs of step
    # k-1 before sending step k's inputs).
    if e2e_steps > 0:
        import ctypes as C
        import torch
        M = sv.M
        fields0 = [sv.get_fields(b) for b in range(B)]
        sv.close()
        Lm = importlib.import_module(f"{PKG}._lib")
        dp = C.POINTER(C.c_double)
        lib = Lm.lib()
        bounds = np.linspace(0, B, e2e_parts + 1).astype(int)
        parts = []
        for k in range(e2e_parts):
            lo, hi = int(bounds[k]), int(bounds[k + 1])
            # the parts run side by side: launch forms tuned on one part alone would not be the
            # fastest with the other parts in flight, so they keep the heuristic forms
            psv = srn.Solver(surfaces[lo:hi], precision=precision, device=device, noise="device", autotune=False)
            for j, b in enumerate(range(lo, hi)):
                if init[b][1] is not None:
                    psv.set_masks(init[b][1], j)
                psv.set_iteration(start_iteration(surfaces[b]) + warmup, j)
                psv.set_rng((11 + b, 22, 33), j)
            w_in = torch.empty((hi - lo, 14, M), dtype=torch.float64, pin_memory=True).numpy()
            w_out = torch.empty((hi - lo, 14, M), dtype=torch.float64, pin_memory=True).numpy()
            phi_host = torch.empty((hi - lo, 14, M), dtype=torch.float64, pin_memory=True).numpy()
            for j, b in enumerate(range(lo, hi)):
                w_in[j] = fields0[b]
            parts.append((psv, (w_in, w_out), phi_host, (Lm.CIterOut * (hi - lo))()))

        def enqueue(part):
            psv, (w_in, w_out), phi_host, _ = part
            Lm.check(lib.scft_set_fields_all_async(psv._h, w_in.ctypes.data_as(dp)), "set_fields_all_async")
            Lm.check(lib.scft_iterate_async(psv._h, 1), "iterate_async")
            Lm.check(lib.scft_get_fields_all_async(psv._h, w_out.ctypes.data_as(dp)), "get_fields_all_async")
            Lm.check(lib.scft_get_densities_all_async(psv._h, phi_host.ctypes.data_as(dp)), "get_densities_all_async")

        def wait(part):
            Lm.check(lib.scft_iterate_wait(part[0]._h, part[3]), "iterate_wait")

        for part in parts:  # one untimed round: graph capture, first touch
            enqueue(part)
        for part in parts:
            wait(part)
        sync()
        t0 = time.perf_counter()
        for part in parts:
            enqueue(part)
        for _ in range(e2e_steps - 1):
            for part in parts:
                wait(part)
                enqueue(part)
        for part in parts:
            wait(part)
        sync()
        e2e = time.perf_counter() - t0
        for part in parts:
            part[0].close()
        res["e2e"] = {"value": B * e2e_steps / e2e, "unit": "instance-iterations/s",
                      "h2d_bytes_per_step": B * 14 * M * 8,
                      "d2h_bytes_per_step": B * (14 + 14) * M * 8 + B * C.sizeof(Lm.CIterOut),
                      "contexts": e2e_parts, "steps": e2e_steps}
        return res
    sv.close()
    return res


def _sweep_form(sw, surfaces, inputs, precision: str, rms_tol: float, max_iter: int, sync):
    """One form of the droplet sweep run to the end (every instance converged
    or at max_iter), timed from the batch's first iteration to its last."""
    with sw.make_batch(surfaces, inputs, precision, rms_tol) as b:
        sync()
        t0 = time.perf_counter()
        res = b.run(max_iter, chunk=200)
        sync()
        wall = time.perf_counter() - t0
        groups = b.groups
    its = np.array([r.iterations for r in res])
    conv = int(sum(r.converged for r in res))
    by_shape = {}
    for s, r in zip(surfaces, res):
        nx, _, nz = s.grid()
        d = by_shape.setdefault(f"{nx}x{nz}", {"instances": 0, "converged": 0, "final_rms": []})
        d["instances"] += 1
        d["converged"] += int(r.converged)
        d["final_rms"].append(float(r.rms))
    for d in by_shape.values():
        v = np.array(d.pop("final_rms"))
        d["final_rms_median"] = float(np.median(v))
        d["final_rms_min"] = float(v.min())
        d["final_rms_max"] = float(v.max())
    return {"instances": len(res), "groups": groups, "converged": conv, "wall_s": wall,
            "solves_per_hour": conv * 3600.0 / wall, "iterations_median": float(np.median(its)),
            "iterations_max": int(its.max()), "instance_iterations_per_s": float(its.sum()) / wall,
            "nonfinite": int(sum(r.status != 0 for r in res)), "by_shape": by_shape,
            "final_rms": [float(r.rms) for r in res], "final_free_energy": [float(r.free_energy) for r in res]}


SWEEP_FORMS = ("fp32", "fp64", "fp32x2", "finish_fp32x2", "finish_fp64")


def measure_sweep(srn, n: int, rms_tol: float, max_iter: int, subset: int, device: int, sync,
                  keep_points: bool = False, forms=SWEEP_FORMS):
    """The 2D droplet sweep (n x n chi points, uneven grids and NS, seeded
    droplet starts) run to RMS < rms_tol or max_iter, every form timed to the
    end: converged solves/hour = converged instances / wall time.
    fp32: the precision form on all n x n points. subset: points on a diagonal
    walk of the chi grid in both forms, the plain FP64 form and the precision
    form on the same instances, the same start and the same stop rule; their
    ratio is read against the >= 5x target. subset >= n*n takes every point.
    forms: which of SWEEP_FORMS run on the subset (the finishing forms and the
    double-float form alone only below the FP32 floor)."""
    sw = importlib.import_module(f"{PKG}.sweep")
    surfaces = srn.configs.sweep_surfaces(n, seed=3, sizes=sw.SWEEP_SIZES, ns_range=(64, 128))
    inputs = sw.sweep_inputs(surfaces)
    full = _sweep_form(sw, surfaces, inputs, "fp32", rms_tol, max_iter, sync)
    full_F, full_rms = list(full["final_free_energy"]), list(full["final_rms"])
    if not keep_points:
        full.pop("final_rms")
        full.pop("final_free_energy")
    out = {"rms_tol": rms_tol, "max_iter": max_iter, "fp32": full}
    if subset > 0:
        # spread over both chi axes: point j sits in row j*n/subset of the grid,
        # column j mod n (a diagonal walk), so every chi_AB and chi_AC band is in
        idx = sorted({(j * n // subset) * n + (j % n) for j in range(subset)} & set(range(len(surfaces))))
        ss = [surfaces[i] for i in idx]
        si = [inputs[i] for i in idx]
        full_set = len(idx) == len(surfaces)
        f32 = full if full_set else _sweep_form(sw, ss, si, "fp32", rms_tol, max_iter, sync)
        f32_F = full_F if full_set else list(f32["final_free_energy"])
        f32_conv = [r < rms_tol for r in (full_rms if full_set else f32["final_rms"])]
        sub = {"points": "all" if full_set else idx, "fp32": f32,
               "basis": "converged instances / wall time to the end, every form on the same instances"}
        ran = [f32]
        f64 = None
        if "fp64" in forms:
            f64 = _sweep_form(sw, ss, si, "fp64", rms_tol, max_iter, sync)
            f64_F = list(f64["final_free_energy"])
            f64_conv = [r < rms_tol for r in f64["final_rms"]]
            both = [k for k in range(len(ss)) if f64_conv[k] and f32_conv[k]]
            sub["fp32_vs_fp64_converged_in_both"] = len(both)
            sub["fp32_vs_fp64_max_rel_free_energy_diff"] = max(
                (abs(f32_F[k] - f64_F[k]) / abs(f64_F[k]) for k in both), default=None)
            sub["fp64_plain"] = f64
            sub["solves_per_hour_ratio_fp32_over_fp64"] = (f32["solves_per_hour"] / f64["solves_per_hour"]
                                                           if f64["solves_per_hour"] > 0 else None)
            ran.append(f64)
        if rms_tol < sw.SWITCH_RMS and "fp32x2" in forms:
            # the double-float form alone, from the start: its per-iteration cost against FP64
            sub["fp32x2"] = _sweep_form(sw, ss, si, "fp32x2", rms_tol, max_iter, sync)
            ran.append(sub["fp32x2"])
        if not keep_points:
            for f in ran:
                f.pop("final_rms", None)
                f.pop("final_free_energy", None)
        out["subset"] = sub
        if rms_tol < sw.SWITCH_RMS:
            # below the FP32 floor: the precision form hands over on its floor, to the
            # double-float form (the library's finish) and, for comparison, to plain FP64
            for finish in ("fp32x2", "fp64"):
                if f"finish_{finish}" not in forms:
                    continue
                sync()
                res, wall, wall32 = sw.run_finished(ss, si, rms_tol, max_iter, finish=finish)
                sync()
                conv = int(sum(r.converged for r in res))
                fin = {"handover": f"RMS < {sw.SWITCH_RMS:g} and falling by less than {1 - sw.STALL_GAIN:g} over "
                                   f"{sw.STALL_ROUND} iterations, or RMS < {sw.FLOOR_RMS:g}; max_iter per instance "
                                   f"over both phases",
                       "converged": conv, "wall_s": wall, "fp32_phase_s": wall32,
                       "solves_per_hour": conv * 3600.0 / wall,
                       "iterations_median": float(np.median([r.iterations for r in res])),
                       "fp32_iterations_median": float(np.median([r.iterations_fp32 for r in res]))}
                if keep_points:
                    fin["final_rms"] = [float(r.rms) for r in res]
                    fin["final_free_energy"] = [float(r.free_energy) for r in res]
                if f64 is not None:
                    # converged in both: the finish form's free energy against the plain FP64 form's
                    both = [k for k, r in enumerate(res) if r.converged and f64_conv[k]]
                    fin["converged_in_both"] = len(both)
                    fin["max_rel_free_energy_diff_vs_fp64"] = max(
                        (abs(res[k].free_energy - f64_F[k]) / abs(f64_F[k]) for k in both), default=None)
                out["subset"][f"fp32_{finish}_finish"] = fin
                if f64 is not None:
                    out["subset"][f"solves_per_hour_ratio_{finish}_finish_over_fp64"] = (
                        fin["solves_per_hour"] / f64["solves_per_hour"] if f64["solves_per_hour"] > 0 else None)
    return out


def _pass_stats(serve, done, wall, classes):
    st = serve.latency_stats(done, wall)
    by = {}
    for k in classes:
        cs = [c for c in done if (c.cls, c.precision) == k]
        if cs:
            lat = np.array([c.latency for c in cs])
            by[f"{k[0]}/{k[1]}"] = {"requests": len(cs), "converged": int(sum(c.converged for c in cs)),
                                    "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                                    "iterations_median": float(np.median([c.iterations for c in cs]))}
    st.update({"wall_s": wall, "by_class": by})
    return st


def measure_serving(srn, n_requests: int, rate_hz: float, rms_tol: float, max_iter: int, device: int,
                    winners: int = 4):
    """Poisson streams of phase-diagram solve requests over 3 planes x 24x24
    (chi_AB N, chi_AC N) points: 70% 2D 192x96 thin film (one in five of those in
    the plain FP64 form), 30% 3D 64^3 bulk blend, NS = 100; slots from a
    device-memory budget. The first pass starts from synthetic seeds (lamellar /
    cylinder / disordered); the second pass is the phase-diagram workflow's
    steady state: every request sits next to a first-pass point (one grid step
    in chi_AB or chi_AC, or the next plane) and starts from that point's final
    field. p50/p99 time from arrival to completion for both passes."""
    serve = importlib.import_module(f"{PKG}.serve")
    cfg = srn.configs
    rng = np.random.default_rng(7)
    chi_ab, chi_ac = cfg.chi_axes(24)
    ft = cfg.film_point(20.0, 40.0, cfg.PLANES[0], ns=100)
    bt = cfg.bulk3d_point(20.0, 40.0, cfg.PLANES[0], ns=100)
    kinds = ("lamellar", "cylinder", "disordered")

    def surface(cls, pl, i, j):
        plane = cfg.PLANES[pl]
        if cls == "film2d":
            return cfg.film_point(float(chi_ab[i]), float(chi_ac[j]), plane, ns=100)
        return cfg.bulk3d_point(float(chi_ab[i]), float(chi_ac[j]), plane, ns=100)

    reqs = []
    t = 0.0
    for r in range(n_requests):
        t += float(rng.exponential(1.0 / rate_hz))
        pl, i, j = int(rng.integers(3)), int(rng.integers(24)), int(rng.integers(24))
        kind = kinds[int(rng.integers(3))]
        cls = "film2d" if rng.random() < 0.7 else "bulk3d"
        prec = "fp64" if cls == "film2d" and rng.random() < 0.2 else "fp32"
        s = surface(cls, pl, i, j)
        reqs.append(serve.Request(rid=r, cls=cls, surface=s, w14=cfg.seed_fields(s, kind, seed=r),
                                  mask3=cfg.substrate_mask(s) if cls == "film2d" else None, precision=prec,
                                  arrival=t, key=(cls, pl, i, j), seed=(r, 5, 7)))
    budget = 24 << 30  # device memory the pools may hold
    slots = {("film2d", "fp32"): serve.slots_for_budget(ft, "fp32", budget // 2, max_slots=64),
             ("film2d", "fp64"): serve.slots_for_budget(ft, "fp64", budget // 6, max_slots=16),
             ("bulk3d", "fp32"): serve.slots_for_budget(bt, "fp32", budget // 3, max_slots=16)}
    tmpl = {"film2d": ft, "bulk3d": bt}
    chunks = {"film2d": 100, "bulk3d": 10}  # about a quarter second of device time per round
    pools = {k: serve.Pool(k[0], tmpl[k[0]], v, k[1], chunk=chunks[k[0]]) for k, v in slots.items()}
    server = serve.Server(pools, rms_tol=rms_tol, max_iter=max_iter, chunk=50, keep_fields=True)
    t0 = time.perf_counter()
    first = server.run(reqs)
    wall1 = time.perf_counter() - t0
    # second pass: neighbours of the first-pass points, seeded with their final fields
    reqs2 = []
    t = 0.0
    for r, c in enumerate(sorted(first, key=lambda c: c.rid)):
        cls, pl, i, j = c.key
        t += float(rng.exponential(1.0 / rate_hz))
        move = int(rng.integers(3))
        if move == 0:
            i = i + 1 if i + 1 < 24 else i - 1
        elif move == 1:
            j = j + 1 if j + 1 < 24 else j - 1
        else:
            pl = (pl + 1) % 3
        s = surface(cls, pl, i, j)
        reqs2.append(serve.Request(rid=1000 + r, cls=cls, surface=s, w14=c.fields,
                                   mask3=cfg.substrate_mask(s) if cls == "film2d" else None, precision=c.precision,
                                   arrival=t, key=(cls, pl, i, j), seed=(r, 9, 7)))
    t0 = time.perf_counter()
    second = server.run(reqs2)
    wall2 = time.perf_counter() - t0
    st = _pass_stats(serve, second, wall2, slots)
    st.update({"pass": "neighbour-seeded (second pass)", "rate_hz": rate_hz, "rms_tol": rms_tol,
               "max_iter": max_iter, "slots": {f"{k[0]}/{k[1]}": v for k, v in slots.items()},
               "first_pass": _pass_stats(serve, first, wall1, slots)})
    if winners > 1:
        st["winners"] = winner_check(serve, server, second, surface, cfg, winners)
    server.close()
    return st


def winner_check(serve, server, done, surface, cfg, k: int) -> dict:
    """Lowest-F winners of the FP32 form against the plain FP64 form, after the
    serving passes (not part of their timing). Up to k converged FP32 thin-film
    results of the second pass give k points and k structures; every structure
    is relaxed at every other point in FP32 (the phase-diagram trial, same
    tolerance and iteration cap as the stream). Both forms then evaluate the
    free energy of every converged structure on the same fields (one iteration
    each: the reference's F uses the fields before the update), and each
    point's lowest-F structure is compared between the two forms. Structures
    whose FP32 free energies lie within 1e-6 relative of the winner's are the
    same structure to FP32 accuracy and count as ties."""
    films = [c for c in sorted(done, key=lambda c: c.rid)
             if c.cls == "film2d" and c.precision == "fp32" and c.converged and c.fields is not None][:k]
    k = len(films)
    if k < 2:
        return {"points": k, "compared": 0, "note": "fewer than two converged FP32 thin-film results"}
    surf = [surface(c.key[0], c.key[1], c.key[2], c.key[3]) for c in films]
    mk = [cfg.substrate_mask(s) for s in surf]
    rid = 100000
    reqs = []
    for a in range(k):
        for b in range(k):
            if a != b:
                rid += 1
                reqs.append(serve.Request(rid=rid, cls="film2d", surface=surf[a], w14=films[b].fields, mask3=mk[a],
                                          precision="fp32", key=(a, b), seed=(a, b, 3)))
    keep = server.keep_fields
    server.keep_fields = True
    try:
        relaxed = {(a, a): (films[a].converged, films[a].fields) for a in range(k)}
        for c in server.run(reqs, realtime=False):
            relaxed[c.key] = (c.converged and np.isfinite(c.free_energy), c.fields)
    finally:
        server.keep_fields = keep
    keys = sorted(key for key, (conv, _) in relaxed.items() if conv)
    Solver = importlib.import_module(PKG).Solver
    F = {}
    for prec in ("fp32", "fp64"):
        with Solver([surf[a] for a, _ in keys], precision=prec) as sv:
            for n, (a, b) in enumerate(keys):
                sv.set_fields(relaxed[(a, b)][1], n)
                sv.set_masks(mk[a], n)
                sv.set_iteration(1, n)
            out = sv.iterate(1)[0]
            F[prec] = {key: out[n].free_energy for n, key in enumerate(keys)}
    compared = agree = ties = 0
    max_rel = max(abs(F["fp32"][key] - F["fp64"][key]) / abs(F["fp64"][key]) for key in keys)
    for a in range(k):
        cand = [b for (a2, b) in keys if a2 == a]
        if len(cand) < 2:
            continue
        compared += 1
        w32 = min(cand, key=lambda b: F["fp32"][(a, b)])
        w64 = min(cand, key=lambda b: F["fp64"][(a, b)])
        if w32 == w64:
            agree += 1
        elif abs(F["fp32"][(a, w64)] - F["fp32"][(a, w32)]) <= 1e-6 * abs(F["fp32"][(a, w32)]):
            ties += 1
    return {"points": k, "fp32_trials": len(reqs), "structures_evaluated": len(keys), "compared": compared,
            "same_winner": agree, "ties_within_1e-6": ties, "different_winner": compared - agree - ties,
            "max_rel_dF_fp32_vs_fp64": max_rel}


def cpu_sample(surfaces, threads: int, iters: int):
    """The CPU restatement of SCFT.c, one instance per thread (ctypes drops the GIL)."""
    srn = importlib.import_module(PKG)
    from oracle.oracle import Oracle
    work = []
    for t in range(threads):
        s = surfaces[t % len(surfaces)]
        w, m = initial_fields(srn, s, 1000 + t)
        o = Oracle(s)
        o.set_fields(w)
        if m is not None:
            o.set_masks(m)
        o.set_iter(1)
        work.append(o)
    times = [0.0] * threads

    def go(k):
        t0 = time.perf_counter()
        work[k].iterate(iters)
        times[k] = time.perf_counter() - t0

    t0 = time.perf_counter()
    th = [threading.Thread(target=go, args=(k,)) for k in range(threads)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    wall = time.perf_counter() - t0
    for o in work:
        o.close()
    return threads * iters / wall, wall


def run_reference(args, rank, world):
    if rank != 0:
        return
    srn = importlib.import_module(PKG)
    surfaces = workload_surfaces(srn, args.workload, args.batch)
    threads = args.cpu_threads or os.cpu_count() or 1
    warmup = args.warmup if args.ref_max_steps <= 0 else min(args.warmup, args.ref_max_steps)
    steps = args.steps if args.ref_max_steps <= 0 else min(args.steps, args.ref_max_steps)
    for _ in range(warmup):
        cpu_sample(surfaces, threads, 1)
    t_all = 0.0
    for _ in range(steps):
        _, wall = cpu_sample(surfaces, threads, 1)
        t_all += wall
    value = threads * steps / t_all
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "instance-iterations/s",
        "n_gpus": world, "steps": steps, "warmup": warmup, "ms_per_step": t_all * 1e3 / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": workload_data(args.workload),
        "config": workload_config(args, surfaces),
        "cpu_baseline": {"value": value, "unit": "instance-iterations/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} steps x 1 iteration of {threads} instances, one per host thread "
                                   f"(SCFT.c's algorithm, data layout and FFT code restated "
                                   f"in oracle/)"},
        "e2e": {"value": value, "unit": "instance-iterations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_data(name: str) -> str:
    start = {"film2d": "seeded half-disk droplet fields", "bulk3d": "seeded w noise",
             "bulk2d": "seeded w noise", "blend3d": "seeded w noise"}.get(name, "seeded fields")
    return f"synthetic ({start}, chi sweep)"


def workload_config(args, surfaces):
    s = surfaces[0]
    nx, ny, nz = s.grid()
    start = "seeded droplet start" if s.MASK else "seeded w-noise start"
    sweep = "seeded chi N matrices" if args.workload == "blend3d" else "chi_AB x chi_AC sweep"
    return {"workload": f"{args.workload} {nx}x{ny}x{nz} NS={s.NS} MASK={s.MASK}, {len(surfaces)} instances "
                        f"({sweep}), {start}",
            "instances_per_gpu": len(surfaces), "grid": [nx, ny, nz], "ns": s.NS, "mask": s.MASK,
            "l2": "working set larger than L2 (propagators of all instances)",
            "parallelism": "replicas (one batch per GPU)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="film2d")
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--e2e-parts", type=int, default=8, help="contexts the e2e batch is pipelined over")
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--cpu-iters", type=int, default=5, help="iterations per host thread of the CPU baseline sample")
    ap.add_argument("--ref-max-steps", type=int, default=0,
                    help="cap on the reference arm's timed (and warm-up) steps; 0: run --steps as given")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64", "fp32x2"])
    ap.add_argument("--sweep-n", type=int, default=16, help="n x n chi points of the droplet sweep (0: skip)")
    ap.add_argument("--sweep-tol", type=float, default=1e-4)
    ap.add_argument("--sweep-max-iter", type=int, default=5000)
    ap.add_argument("--sweep-subset", type=int, default=16,
                    help="points of the sweep run in both forms to the end (0: precision form only)")
    ap.add_argument("--sweep-points", action="store_true", help="keep every point's final RMS in the sweep record")
    ap.add_argument("--sweep-forms", default=",".join(SWEEP_FORMS),
                    help="forms run on the sweep subset: fp32, fp64, fp32x2, finish_fp32x2, finish_fp64")
    ap.add_argument("--serve-requests", type=int, default=40, help="requests of the serving stream (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=4.0, help="mean arrivals per second")
    ap.add_argument("--serve-tol", type=float, default=1e-4)
    ap.add_argument("--serve-max-iter", type=int, default=4000)
    ap.add_argument("--serve-winners", type=int, default=4,
                    help="points of the FP32-vs-FP64 lowest-F winner check after serving (0: skip)")
    ap.add_argument("--profile-iters", type=int, default=1, help="iterations of --profile-case")
    ap.add_argument("--profile-case", action="store_true",
                    help="one iteration of one form only (for ncu captures; the iterations sit in a "
                         "profiler range for --profile-from-start off); prints no bench line")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    rank, world, local = dist_env()

    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    srn = importlib.import_module(PKG)
    importlib.import_module(f"{PKG}.build").build()
    import torch
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist

    def sync():
        torch.cuda.synchronize()
        if pg is not None:
            pg.barrier()

    surfaces = workload_surfaces(srn, args.workload, args.batch)
    if args.profile_case:
        sv = srn.Solver(surfaces, precision=args.precision, device=local, noise="device")
        for b, s in enumerate(surfaces):
            w, m = initial_fields(srn, s, 1000 + b)
            sv.set_fields(w, b)
            if m is not None:
                sv.set_masks(m, b)
            sv.set_iteration(start_iteration(s), b)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        out = sv.iterate(args.profile_iters)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print(f"profile case: {len(surfaces)} instances, {args.profile_iters} iteration(s), "
              f"F[0] = {out[-1][0].free_energy:.12f}")
        sv.close()
        return
    f32 = measure_form(srn, surfaces, "fp32", args.steps, args.warmup, local, sync, args.e2e_steps, args.e2e_parts)
    f64 = measure_form(srn, surfaces, "fp64", args.fp64_steps, 1, local, sync, 0)
    ms, ms64 = max_over_ranks(pg, [f32["ms_per_step"], f64["ms_per_step"]], "cuda")
    B = len(surfaces)
    value = job_rate(world, B, ms)
    peaks = json.loads(PEAKS.read_text()) if PEAKS.exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    traffic = None
    if TRAFFIC.exists():
        tr = json.loads(TRAFFIC.read_text()).get(args.workload, {})
        if tr.get("instances") == len(surfaces):
            traffic = tr.get("traffic_bytes_per_launch")
    line = {
        "metric": METRIC, "value": value, "unit": "instance-iterations/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 propagators, f64 densities/Q/free energy/update",
        "data": workload_data(args.workload),
        "config": workload_config(args, surfaces),
        "e2e": f32.get("e2e"),
        "gpu_launches": f32["gpu_launches"],
        "clocks": f32["clocks"],
        "roofline": {"bound": "hbm", "achieved": f32["achieved_gbs"], "peak": peak, "unit": "GB/s",
                     "frac": f32["achieved_gbs"] / peak, "traffic": traffic,
                     "peak_source": "measured" if PEAKS.exists() else "fallback",
                     "kernel": f32["kernel"],
                     "algorithmic_bytes_per_launch": f32["algorithmic_bytes_per_step"] / f32["prop_launches_per_step"],
                     "launch_ms": f32["prop_ms_per_step"] / f32["prop_launches_per_step"]},
        "fp64_plain": {"value": job_rate(world, B, ms64), "ms_per_step": ms64, "steps": args.fp64_steps,
                       "achieved_gbs": f64["achieved_gbs"], "frac": f64["achieved_gbs"] / peak,
                       "prop_ms_per_step": f64["prop_ms_per_step"], "clocks": f64["clocks"]},
        "detail": {"fp32_prop_ms_per_step": f32["prop_ms_per_step"], "fp32_wall_ms_per_step": f32["wall_ms_per_step"],
                   "contour_steps_per_instance_iteration": f32["contour_steps_per_instance_iteration"],
                   "device_bytes_fp32": f32["device_bytes"],
                   "fp32_threads_per_line": f32["threads_per_line"]},
    }
    # the sweep and the serving stream are single-GPU measurements (replicas add nothing to them)
    if world > 1:
        args.sweep_n = args.serve_requests = 0
    if args.sweep_n > 0:
        line["sweep"] = measure_sweep(srn, args.sweep_n, args.sweep_tol, args.sweep_max_iter, args.sweep_subset,
                                      local, sync, keep_points=args.sweep_points,
                                      forms=tuple(f for f in args.sweep_forms.split(",") if f))
    if args.serve_requests > 0:
        line["serving"] = measure_serving(srn, args.serve_requests, args.serve_rate, args.serve_tol,
                                          args.serve_max_iter, local, args.serve_winners)
    if rank == 0 and not args.no_cpu:
        threads = args.cpu_threads or os.cpu_count() or 1
        rate, wall = cpu_sample(surfaces, threads, args.cpu_iters)
        line["cpu_baseline"] = {"value": rate, "unit": "instance-iterations/s", "cores": threads, "kind": "port",
                                "sample": f"{args.cpu_iters} iteration(s) of {threads} instances, one per host "
                                          f"thread, {wall:.1f} s (SCFT.c's algorithm restated in oracle/)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
