"""Python face of the GB300 SCFT library, shaped like the reference's run.

``Solver`` holds one library context (one or many instances that share grid and
contour counts) and exposes the same steps SCFT.c's main() takes: derive the
run parameters, load restart fields / masks / RNG state, run iterations,
read fields and densities back, and write the reference's output files.
All compute goes through libscft_gb300.so; nothing here computes SCFT
quantities itself.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
from typing import List, Optional, Sequence

import numpy as np

from . import _lib as L
from .surface import Surface

SPECIES = ["dbk1", "dbk2", "dbk3", "dbk4"] + [f"homo_{x}" for x in "ABCDEFGHIJ"] + ["S1", "S2", "S3"]


@dataclasses.dataclass
class Derived:
    """scft_derived as Python values (SCFT.c:84-396, :718-733)."""

    c: L.CDerived
    status: int

    def __getattr__(self, name):
        v = getattr(self.c, name)
        if isinstance(v, C.Array):
            a = np.ctypeslib.as_array(v)
            return a.copy()
        return v

    @property
    def grid(self):
        return self.c.nx, self.c.ny, self.c.nz

    @property
    def M(self) -> int:
        return int(self.c.m)


def derive(s: Surface) -> Derived:
    cs = L.CSurface.from_surface(s)
    d = L.CDerived()
    rc = L.lib().scft_derive(C.byref(cs), C.byref(d))
    if rc not in (L.SCFT_OK, -5):
        L.check(rc, "scft_derive")
    return Derived(d, rc)


@dataclasses.dataclass
class IterOut:
    iter: int
    free_energy: float
    rms: float
    mf: float
    mu: np.ndarray
    q: np.ndarray
    status: int
    converged: int = 0

    @classmethod
    def from_c(cls, r: L.CIterOut) -> "IterOut":
        return cls(int(r.iter), float(r.free_energy), float(r.rms), float(r.mf), np.array(r.mu[:]), np.array(r.q[:]),
                   int(r.status), int(r.converged))

    def to_c(self) -> L.CIterOut:
        r = L.CIterOut()
        r.iter, r.free_energy, r.rms, r.mf, r.status = self.iter, self.free_energy, self.rms, self.mf, self.status
        r.converged = self.converged
        for k in range(L.NSP):
            r.mu[k] = self.mu[k]
            r.q[k] = self.q[k]
        return r


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _us3(seed) -> C.Array:
    return (C.c_ushort * 3)(*[int(x) for x in seed])


class Solver:
    """One GPU context for ``len(surfaces)`` SCFT instances of one shape.

    precision: "fp64" (plain form, the drop-in), "fp32" (FP32 propagators,
    FP64 densities/Q/free energy/update) or "fp32x2" (propagators in
    double-float arithmetic, pairs of FP32 with ~48 significant bits, FP64
    reductions: the finishing form below the FP32 form's RMS floor).
    noise: "host" (the caller passes the drand48 draws to iterate) or "device"
    (the library replays the drand48 stream itself from set_rng's state).
    """

    def __init__(self, surfaces: Surface | Sequence[Surface], precision: str = "fp64", device: int = 0,
                 use_graph: bool = False, kernel_path: str = "auto", noise: str = "host", autotune: bool = True):
        if isinstance(surfaces, Surface):
            surfaces = [surfaces]
        self.surfaces = list(surfaces)
        self.B = len(self.surfaces)
        arr = (L.CSurface * self.B)(*[L.CSurface.from_surface(s) for s in self.surfaces])
        opt = L.COptions()
        L.lib().scft_options_default(C.byref(opt))
        opt.precision = {"fp64": L.PREC_FP64, "fp32": L.PREC_FP32, "fp32x2": L.PREC_FP32X2}[precision]
        opt.device = device
        opt.use_graph = int(bool(use_graph))
        opt.n_instances = self.B
        opt.kernel_path = {"auto": 0, "passes": 1}[kernel_path]
        opt.noise_mode = {"host": L.NOISE_HOST, "device": L.NOISE_DRAND48}[noise]
        opt.autotune = int(bool(autotune))
        self.noise_mode = noise
        self.precision = precision
        h = C.c_void_p()
        L.check(L.lib().scft_ctx_create(arr, C.byref(opt), C.byref(h)), "scft_ctx_create")
        self._h = h
        self.derived = []
        for b in range(self.B):
            d = L.CDerived()
            L.check(L.lib().scft_ctx_derived(h, b, C.byref(d)), "scft_ctx_derived")
            self.derived.append(Derived(d, 0))
        self.M = self.derived[0].M
        self.grid = self.derived[0].grid

    # ------------------------------------------------------------ lifecycle
    def close(self):
        if getattr(self, "_h", None):
            L.lib().scft_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def device_bytes(self) -> int:
        return int(L.lib().scft_ctx_device_bytes(self._h))

    # --------------------------------------------------------------- state
    def set_fields(self, w14: np.ndarray, instance: int = 0):
        w14 = np.ascontiguousarray(w14, dtype=np.float64).reshape(14, self.M)
        L.check(L.lib().scft_set_fields(self._h, instance, _dp(w14)), "scft_set_fields")

    def set_masks(self, mask3: np.ndarray, instance: int = 0):
        mask3 = np.ascontiguousarray(mask3, dtype=np.float64).reshape(3, self.M)
        L.check(L.lib().scft_set_masks(self._h, instance, _dp(mask3)), "scft_set_masks")

    def set_iteration(self, it: int, instance: int = 0):
        L.check(L.lib().scft_set_iteration(self._h, instance, int(it)), "scft_set_iteration")

    def set_rng(self, seed, instance: int = 0):
        L.check(L.lib().scft_set_rng(self._h, instance, _us3(seed)), "scft_set_rng")

    def get_rng(self, instance: int = 0):
        s = (C.c_ushort * 3)()
        L.check(L.lib().scft_get_rng(self._h, instance, s), "scft_get_rng")
        return tuple(int(x) for x in s)

    def iterate(self, n: int = 1, noise: Optional[np.ndarray] = None) -> List[List[IterOut]]:
        """Run n iterations on every instance; returns out[iteration][instance]."""
        outs = (L.CIterOut * (n * self.B))()
        nd = None
        if noise is not None:
            noise = np.ascontiguousarray(noise, dtype=np.float64)
            nd = _dp(noise)
        L.check(L.lib().scft_iterate(self._h, n, nd, outs), "scft_iterate")
        return [[IterOut.from_c(outs[k * self.B + b]) for b in range(self.B)] for k in range(n)]

    def set_surface(self, instance: int, surface: Surface):
        """Give a slot new parameters (same grid and composition; NS within the slot's capacity)."""
        cs = L.CSurface.from_surface(surface)
        L.check(L.lib().scft_set_surface(self._h, instance, C.byref(cs)), "scft_set_surface")
        self.surfaces[instance] = surface
        d = L.CDerived()
        L.check(L.lib().scft_ctx_derived(self._h, instance, C.byref(d)), "scft_ctx_derived")
        self.derived[instance] = Derived(d, 0)

    def freeze(self, instance: int):
        """Idle a slot: later iterations skip it until set_iteration re-arms it."""
        L.check(L.lib().scft_freeze(self._h, instance), "scft_freeze")

    def set_stop(self, rms_tol: float, instance: Optional[int] = None):
        """Freeze an instance (every instance if None) once RMS(phi_tot-1) < rms_tol."""
        for b in (range(self.B) if instance is None else [instance]):
            L.check(L.lib().scft_set_stop(self._h, b, float(rms_tol)), "scft_set_stop")

    def iterate_async(self, n: int):
        """Enqueue n <= 256 iterations (device noise or no noise) without waiting."""
        L.check(L.lib().scft_iterate_async(self._h, int(n)), "scft_iterate_async")
        self._pending = int(n)

    def iterate_ready(self) -> bool:
        """True once the enqueued iterations have finished (never blocks)."""
        r = L.lib().scft_iterate_ready(self._h)
        if r < 0:
            L.check(r, "scft_iterate_ready")
        return bool(r)

    def iterate_wait(self, allow_nonfinite: bool = False) -> List[List[IterOut]]:
        """Records of the enqueued iterations, [iteration][instance].
        allow_nonfinite: an instance that turned non-finite does not raise;
        its records carry status SCFT_ERR_NONFINITE and the others are intact."""
        n = getattr(self, "_pending", 0)
        outs = (L.CIterOut * max(1, n * self.B))()
        rc = L.lib().scft_iterate_wait(self._h, outs)
        self._pending = 0
        if not (allow_nonfinite and rc == L.ERR_NONFINITE):
            L.check(rc, "scft_iterate_wait")
        return [[IterOut.from_c(outs[k * self.B + b]) for b in range(self.B)] for k in range(n)]

    def get_fields(self, instance: int = 0) -> np.ndarray:
        w = np.empty((14, self.M))
        L.check(L.lib().scft_get_fields(self._h, instance, _dp(w)), "scft_get_fields")
        return w

    def get_densities(self, instance: int = 0):
        phi = np.empty((13, self.M))
        tot = np.empty(self.M)
        L.check(L.lib().scft_get_densities(self._h, instance, _dp(phi), _dp(tot)), "scft_get_densities")
        return phi, tot

    def propagate(self, q0: np.ndarray, w: np.ndarray, steps: int) -> np.ndarray:
        """funPDESolver's contour loop for one block (unit entry point)."""
        q0 = np.ascontiguousarray(q0, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        out = np.empty((steps + 1, self.M))
        L.check(L.lib().scft_propagate(self._h, _dp(q0), _dp(w), int(steps), _dp(out)), "scft_propagate")
        return out

    def density(self, qf: np.ndarray, qb: np.ndarray, start: int, stop: int, q: float) -> np.ndarray:
        """funMultiplyQs + funDensity for one block (unit entry point)."""
        qf = np.ascontiguousarray(qf, dtype=np.float64)
        qb = np.ascontiguousarray(qb, dtype=np.float64)
        n = qf.shape[0]
        out = np.empty(self.M)
        L.check(L.lib().scft_density(self._h, _dp(qf), _dp(qb), int(n), int(start), int(stop), float(q), _dp(out)),
                "scft_density")
        return out

    def enable_timing(self, on: bool = True):
        L.check(L.lib().scft_enable_timing(self._h, int(on)), "scft_enable_timing")

    def timing(self) -> dict:
        t = L.CTiming()
        L.check(L.lib().scft_get_timing(self._h, C.byref(t)), "scft_get_timing")
        return {"total_ms": t.total_ms, "prop_ms": t.prop_ms, "prop_launches": t.prop_launches,
                "kernel_launches": t.kernel_launches, "fused_chain": int(t.fused_chain),
                "threads_per_line": int(t.threads_per_line)}


# ----------------------------------------------------------------- host side
def noise_fill(state, d: Derived, out: bool = True):
    """One iteration of the reference's noise draws (funGaussDev order).

    Returns (noise[n_active, M] or None, new_state)."""
    st = _us3(state)
    arr = np.empty((d.c.n_active, d.M)) if out else None
    L.check(L.lib().scft_noise_fill(st, C.byref(d.c), _dp(arr) if out else None), "scft_noise_fill")
    return arr, tuple(int(x) for x in st)


def _dir(path) -> bytes:
    return os.fsencode(str(path)) if path is not None else None


def read_counter(path) -> int:
    v = C.c_ulong()
    L.check(L.lib().scft_read_counter(_dir(path), C.byref(v)), "scft_read_counter")
    return int(v.value)


def read_restart_fields(path, d: Derived) -> np.ndarray:
    w = np.empty((14, d.M))
    L.check(L.lib().scft_read_restart_fields(_dir(path), C.byref(d.c), _dp(w)), "scft_read_restart_fields")
    return w


def read_restart_random(path):
    s = (C.c_ushort * 3)()
    L.check(L.lib().scft_read_restart_random(_dir(path), s), "scft_read_restart_random")
    return tuple(int(x) for x in s)


def read_mask(path, d: Derived) -> np.ndarray:
    m = np.empty((3, d.M))
    L.check(L.lib().scft_read_mask(_dir(path), C.byref(d.c), _dp(m)), "scft_read_mask")
    return m


def write_energies(path, d: Derived, o: IterOut):
    r = o.to_c()
    L.check(L.lib().scft_write_energies(_dir(path), C.byref(d.c), C.byref(r)), "scft_write_energies")


def write_snapshot(path, d: Derived, it: int, phi13: np.ndarray, w14: np.ndarray, seed=None):
    phi13 = np.ascontiguousarray(phi13, dtype=np.float64)
    w14 = np.ascontiguousarray(w14, dtype=np.float64)
    L.check(L.lib().scft_write_snapshot(_dir(path), C.byref(d.c), int(it), _dp(phi13), _dp(w14),
                                        _us3(seed) if seed is not None else None), "scft_write_snapshot")


def write_run_params(path, s: Surface, d: Derived, it: int):
    cs = L.CSurface.from_surface(s)
    L.check(L.lib().scft_write_run_params(_dir(path), C.byref(cs), C.byref(d.c), int(it)), "scft_write_run_params")


def device_memory(device: int = 0):
    """(free, total) bytes of a GPU's memory."""
    f, t = C.c_size_t(0), C.c_size_t(0)
    L.check(L.lib().scft_device_memory(int(device), C.byref(f), C.byref(t)), "scft_device_memory")
    return int(f.value), int(t.value)


#: parameters.h file-name macro -> scft_file_names field
_NAME_FIELD = {"COUNTER": "counter", "DENSITY": "density", "DEVIATIONS": "deviations", "ENERGY": "energy",
               "RESTART_FIELDS": "restart_fields", "RESTART_RANDOM": "restart_random", "RUN_PARAMS": "run_params",
               "W_MASK": "w_mask", "FREE_ENERGY": "free_energy"}


def set_file_names(s: Optional[Surface]):
    """Name the text files after the surface's file-name macros (SCFT.c opens
    them through COUNTER ... FREE_ENERGY, parameters.h:181-190); None restores
    the reference's names. Process-wide, like the reference's compiled-in names."""
    if s is None:
        L.check(L.lib().scft_set_file_names(None), "scft_set_file_names")
        return
    n = L.CFileNames()
    for macro, field in _NAME_FIELD.items():
        v = s.file_name(macro).encode()
        if not v or len(v) >= L.NAME_MAX:
            raise ValueError(f"file name for {macro}: {v!r}")
        setattr(n, field, v)
    L.check(L.lib().scft_set_file_names(C.byref(n)), "scft_set_file_names")


def write_volume_error(path, volume_sum: float):
    L.check(L.lib().scft_write_volume_error(_dir(path), float(volume_sum)), "scft_write_volume_error")


def grid_to_idx(nx, ny, nz):
    """Arrays (i, j, k) of every idx = k + NZ*(j + NY*i)."""
    idx = np.arange(nx * ny * nz)
    return idx // (ny * nz), (idx // nz) % ny, idx % nz
