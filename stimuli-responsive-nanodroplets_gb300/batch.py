"""Batching form over instances of uneven grid sizes (scft_batch_* in the C ABI).

The reference runs one SCFT instance per process for a fixed ITER
(SCFT.c:1088); a parameter sweep there is many processes. ``Batch`` puts the
whole sweep on one GPU: surfaces are grouped by grid (one context, stream,
persistent chain kernel and CUDA graph per group), groups run side by side,
and each instance stops when RMS(phi_tot - 1) falls below its tolerance.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Sequence

import numpy as np

from . import _lib as L
from .solver import _dp, _us3, derive
from .surface import Surface


@dataclass
class BatchResult:
    iterations: int
    iter: int
    free_energy: float
    rms: float
    converged: bool
    status: int


class Batch:
    def __init__(self, surfaces: Sequence[Surface], precision: str = "fp32", device: int = 0, use_graph: bool = True,
                 noise: str = "device", kernel_path: str = "auto"):
        self.surfaces = list(surfaces)
        self.n = len(self.surfaces)
        arr = (L.CSurface * self.n)(*[L.CSurface.from_surface(s) for s in self.surfaces])
        opt = L.COptions()
        L.lib().scft_options_default(C.byref(opt))
        opt.precision = {"fp64": L.PREC_FP64, "fp32": L.PREC_FP32, "fp32x2": L.PREC_FP32X2}[precision]
        opt.device = device
        opt.use_graph = int(bool(use_graph))
        opt.kernel_path = {"auto": 0, "passes": 1}[kernel_path]
        opt.noise_mode = {"host": L.NOISE_HOST, "device": L.NOISE_DRAND48}[noise]
        h = C.c_void_p()
        L.check(L.lib().scft_batch_create(arr, self.n, C.byref(opt), C.byref(h)), "scft_batch_create")
        self._h = h
        self.precision = precision
        self.M = [derive(s).M for s in self.surfaces]

    def close(self):
        if getattr(self, "_h", None):
            L.lib().scft_batch_destroy(self._h)
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
    def groups(self) -> int:
        return int(L.lib().scft_batch_groups(self._h))

    def locate(self, i: int):
        g, s = C.c_int(), C.c_int()
        L.check(L.lib().scft_batch_locate(self._h, i, C.byref(g), C.byref(s)), "scft_batch_locate")
        return g.value, s.value

    def set_fields(self, i: int, w14: np.ndarray):
        w14 = np.ascontiguousarray(w14, dtype=np.float64).reshape(14, self.M[i])
        L.check(L.lib().scft_batch_set_fields(self._h, i, _dp(w14)), "scft_batch_set_fields")

    def set_masks(self, i: int, mask3: np.ndarray):
        mask3 = np.ascontiguousarray(mask3, dtype=np.float64).reshape(3, self.M[i])
        L.check(L.lib().scft_batch_set_masks(self._h, i, _dp(mask3)), "scft_batch_set_masks")

    def set_iteration(self, i: int, it: int):
        L.check(L.lib().scft_batch_set_iteration(self._h, i, int(it)), "scft_batch_set_iteration")

    def set_rng(self, i: int, seed):
        L.check(L.lib().scft_batch_set_rng(self._h, i, _us3(seed)), "scft_batch_set_rng")

    def set_stop(self, i: int, rms_tol: float):
        L.check(L.lib().scft_batch_set_stop(self._h, i, float(rms_tol)), "scft_batch_set_stop")

    def freeze(self, i: int):
        """Stop instance i now; set_iteration re-arms it."""
        L.check(L.lib().scft_batch_freeze(self._h, i), "scft_batch_freeze")

    def get_fields(self, i: int) -> np.ndarray:
        w = np.empty((14, self.M[i]))
        L.check(L.lib().scft_batch_get_fields(self._h, i, _dp(w)), "scft_batch_get_fields")
        return w

    def get_densities(self, i: int):
        phi = np.empty((13, self.M[i]))
        tot = np.empty(self.M[i])
        L.check(L.lib().scft_batch_get_densities(self._h, i, _dp(phi), _dp(tot)), "scft_batch_get_densities")
        return phi, tot

    def run(self, max_iter: int, chunk: int = 100) -> List[BatchResult]:
        res = (L.CBatchResult * self.n)()
        L.check(L.lib().scft_batch_run(self._h, int(max_iter), int(chunk), res), "scft_batch_run")
        return [BatchResult(int(r.iterations), int(r.iter), float(r.free_energy), float(r.rms), bool(r.converged),
                            int(r.status)) for r in res]
