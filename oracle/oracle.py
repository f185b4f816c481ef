"""ctypes binding of the CPU oracle (liboracle.so). TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm may use this module, and only as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import importlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle import build as _build  # noqa: E402

NSPEC = 17
REC = 4 + 2 * NSPEC

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(str(path))
        dp = C.POINTER(C.c_double)
        vp = C.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [vp]
        L.orc_destroy.argtypes = [vp]
        L.orc_m.restype = C.c_long
        L.orc_m.argtypes = [vp]
        L.orc_grid.argtypes = [vp, C.POINTER(C.c_int)]
        L.orc_nactive.restype = C.c_int
        L.orc_nactive.argtypes = [vp]
        for name in ("orc_set_fields", "orc_get_fields", "orc_set_masks"):
            getattr(L, name).argtypes = [vp, dp]
        L.orc_set_iter.argtypes = [vp, C.c_ulong]
        L.orc_set_rng.argtypes = [vp, C.POINTER(C.c_ushort)]
        L.orc_get_rng.argtypes = [vp, C.POINTER(C.c_ushort)]
        L.orc_get_densities.argtypes = [vp, dp, dp]
        L.orc_derived.argtypes = [vp, C.POINTER(C.c_int), dp]
        L.orc_propagate.argtypes = [vp, dp, dp, C.c_int, dp]
        L.orc_density.argtypes = [vp, dp, dp, C.c_int, C.c_int, C.c_int, C.c_double, dp]
        L.orc_iterate.restype = C.c_int
        L.orc_iterate.argtypes = [vp, C.c_int, dp]
        L.orc_surface_size.restype = C.c_size_t
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """The reference algorithm on the CPU for one Surface (runtime parameters)."""

    def __init__(self, surface):
        srn = importlib.import_module("stimuli-responsive-nanodroplets_gb300")
        from importlib import import_module
        L_ = import_module("stimuli-responsive-nanodroplets_gb300._lib")
        self._cs = L_.CSurface.from_surface(surface)
        self._h = lib().orc_create(C.byref(self._cs))
        g = (C.c_int * 3)()
        lib().orc_grid(self._h, g)
        self.grid = tuple(g)
        self.M = int(lib().orc_m(self._h))
        self.n_active = int(lib().orc_nactive(self._h))
        self.surface = surface
        del srn

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_fields(self, w14):
        w14 = np.ascontiguousarray(w14, dtype=np.float64)
        lib().orc_set_fields(self._h, _dp(w14))

    def get_fields(self):
        w = np.empty((14, self.M))
        lib().orc_get_fields(self._h, _dp(w))
        return w

    def set_masks(self, m3):
        m3 = np.ascontiguousarray(m3, dtype=np.float64)
        lib().orc_set_masks(self._h, _dp(m3))

    def set_iter(self, it):
        lib().orc_set_iter(self._h, int(it))

    def set_rng(self, seed):
        lib().orc_set_rng(self._h, (C.c_ushort * 3)(*seed))

    def get_rng(self):
        s = (C.c_ushort * 3)()
        lib().orc_get_rng(self._h, s)
        return tuple(int(x) for x in s)

    def iterate(self, n=1):
        """Returns an (n, 38) array: iter, H, rms, MF, mu[17], Q[17]."""
        rec = np.empty((n, REC))
        lib().orc_iterate(self._h, n, _dp(rec))
        return rec

    def densities(self):
        phi = np.empty((13, self.M))
        tot = np.empty(self.M)
        lib().orc_get_densities(self._h, _dp(phi), _dp(tot))
        return phi, tot

    def derived(self):
        ints = (C.c_int * (5 + 13 + 3 * NSPEC))()
        dbls = (C.c_double * (5 + 13 + 169 + NSPEC))()
        lib().orc_derived(self._h, ints, dbls)
        I = list(ints)
        Dd = list(dbls)
        return {
            "grid": tuple(I[0:3]), "N": I[3], "n_active": I[4], "active": I[5:18],
            "len": I[18::3][:NSPEC], "nsx": I[19::3][:NSPEC], "nsy": I[20::3][:NSPEC],
            "ds": Dd[0], "alpha": Dd[1:4], "coating": Dd[4], "phi_avg": Dd[5:18],
            "chi": np.array(Dd[18:18 + 169]).reshape(13, 13), "alpha_sp": Dd[187:187 + NSPEC],
        }

    def propagate(self, q0, w, steps):
        q0 = np.ascontiguousarray(q0, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        out = np.empty((steps + 1, self.M))
        lib().orc_propagate(self._h, _dp(q0), _dp(w), int(steps), _dp(out))
        return out

    def density(self, qf, qb, start, stop, q):
        """funMultiplyQs + funDensity for one block (qf, qb: [len][M])."""
        qf = np.ascontiguousarray(qf, dtype=np.float64)
        qb = np.ascontiguousarray(qb, dtype=np.float64)
        out = np.empty(self.M)
        lib().orc_density(self._h, _dp(qf), _dp(qb), int(qf.shape[0]), int(start), int(stop), float(q), _dp(out))
        return out
