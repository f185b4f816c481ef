"""ctypes view of include/scft_gpu.h (libscft_gb300.so).

The structs here mirror the C declarations field for field. Loading fails
loudly when the library is missing: there is no Python or CPU fallback for
anything the library computes.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from .surface import FIELDS, Surface

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libscft_gb300.so"

NF = 13
NSP = 17

SCFT_OK = 0
ERR_NONFINITE = -4
ERRORS = {
    -1: "SCFT_ERR_PARAM", -2: "SCFT_ERR_CUDA", -3: "SCFT_ERR_OOM", -4: "SCFT_ERR_NONFINITE",
    -5: "SCFT_ERR_VOLUME", -6: "SCFT_ERR_STATE", -7: "SCFT_ERR_IO", -8: "SCFT_ERR_NODEV",
}
PREC_FP64 = 0
PREC_FP32 = 1
PREC_FP32X2 = 2
NOISE_HOST = 0
NOISE_DRAND48 = 1

D = C.c_double
Arr13 = D * NF


class CSurface(C.Structure):
    _fields_ = [
        ("lx", D), ("ly", D), ("lz", D),
        ("iter", C.c_long), ("d_wrt", C.c_long), ("relaxation", C.c_long), ("d_wrt_energies", C.c_long),
        ("dt_noise", D),
        ("mask", C.c_int), ("enable_seed", C.c_int), ("seed_steps", C.c_int), ("seed_area_delta", C.c_int),
        ("ns", C.c_int), ("pad0", C.c_int),
        ("dr_target", D), ("g1", D),
        ("chi_n", Arr13 * NF),
        ("f_dbk", D * 4), ("len_dbk", D * 4), ("vol_dbk", D * 4),
        ("vol_homo", D * 10), ("len_homo", D * 10),
        ("vol_s", D * 3), ("len_s", D * 3),
    ]

    @classmethod
    def from_surface(cls, s: Surface) -> "CSurface":
        c = cls()
        c.lx, c.ly, c.lz = s.LX, s.LY, s.LZ
        c.iter, c.d_wrt, c.relaxation, c.d_wrt_energies = int(s.ITER), int(s.D_WRT), int(s.RELAXATION), int(
            s.D_WRT_ENERGIES)
        c.dt_noise = s.DT_NOISE
        c.mask, c.enable_seed, c.seed_steps, c.seed_area_delta = int(s.MASK), int(s.ENABLE_SEED), int(
            s.SEED_STEPS), int(s.SEED_AREA_DELTA)
        c.ns = int(s.NS)
        c.dr_target, c.g1 = s.DR_TARGET, s.G1
        tab = s.chi_table()
        for f in range(NF):
            for g in range(NF):
                c.chi_n[f][g] = tab[f][g]
        for k in range(4):
            c.f_dbk[k], c.len_dbk[k], c.vol_dbk[k] = s.F_INPUT_DBK[k], s.LEN_DBK[k], s.VOL_DBK[k]
        for k in range(10):
            c.vol_homo[k], c.len_homo[k] = s.VOL_HOMO[k], s.LEN_HOMO[k]
        for k in range(3):
            c.vol_s[k], c.len_s[k] = s.VOL_S[k], s.LEN_S[k]
        return c


class CDerived(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("n_ext", C.c_int),
        ("m", C.c_long),
        ("ds", D), ("dx", D), ("dy", D), ("dz", D), ("alphax", D), ("alphay", D), ("alphaz", D),
        ("ns_dbk", C.c_int * 4), ("ns_dbk_x", C.c_int * 4), ("ns_dbk_y", C.c_int * 4),
        ("ns_homo", C.c_int * 10), ("ns_s", C.c_int * 3),
        ("alpha_dbk", D * 4), ("alpha_homo", D * 10), ("alpha_s", D * 3),
        ("phi_avg", Arr13), ("chi_eff", Arr13 * NF), ("coating_vol", D),
        ("active", C.c_int * NF), ("n_active", C.c_int),
        ("volume_sum", D), ("volume_ok", C.c_int),
    ]


class COptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("device", C.c_int), ("noise_mode", C.c_int), ("use_graph", C.c_int),
                ("n_instances", C.c_int), ("kernel_path", C.c_int), ("autotune", C.c_int), ("reserved", C.c_int)]


class CIterOut(C.Structure):
    _fields_ = [("iter", C.c_ulong), ("free_energy", D), ("rms", D), ("mf", D), ("mu", D * NSP), ("q", D * NSP),
                ("status", C.c_int), ("converged", C.c_int)]


class CBatchResult(C.Structure):
    _fields_ = [("iterations", C.c_ulong), ("iter", C.c_ulong), ("free_energy", D), ("rms", D),
                ("converged", C.c_int), ("status", C.c_int)]


NAME_MAX = 256
FILE_NAME_FIELDS = ["counter", "density", "deviations", "energy", "restart_fields", "restart_random", "run_params",
                    "w_mask", "free_energy"]


class CFileNames(C.Structure):
    _fields_ = [(n, C.c_char * NAME_MAX) for n in FILE_NAME_FIELDS]


class CTiming(C.Structure):
    _fields_ = [("total_ms", D), ("prop_ms", D), ("prop_launches", C.c_long), ("kernel_launches", C.c_long),
                ("fused_chain", C.c_int), ("threads_per_line", C.c_int)]


_lib = None


def lib() -> C.CDLL:
    """Load libscft_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() (no CPU fallback exists)")
    L = C.CDLL(str(LIB_PATH))
    P, I, UL, VP = C.POINTER, C.c_int, C.c_ulong, C.c_void_p
    dp = P(D)
    us3 = P(C.c_ushort)
    sigs = {
        "scft_derive": (I, [P(CSurface), P(CDerived)]),
        "scft_options_default": (None, [P(COptions)]),
        "scft_ctx_create": (I, [P(CSurface), P(COptions), P(VP)]),
        "scft_ctx_destroy": (I, [VP]),
        "scft_ctx_derived": (I, [VP, I, P(CDerived)]),
        "scft_ctx_device_bytes": (C.c_size_t, [VP]),
        "scft_set_fields": (I, [VP, I, dp]),
        "scft_set_masks": (I, [VP, I, dp]),
        "scft_set_iteration": (I, [VP, I, UL]),
        "scft_set_rng": (I, [VP, I, us3]),
        "scft_get_rng": (I, [VP, I, us3]),
        "scft_iterate": (I, [VP, I, dp, P(CIterOut)]),
        "scft_set_stop": (I, [VP, I, D]),
        "scft_freeze": (I, [VP, I]),
        "scft_set_surface": (I, [VP, I, P(CSurface)]),
        "scft_iterate_async": (I, [VP, I]),
        "scft_iterate_wait": (I, [VP, P(CIterOut)]),
        "scft_iterate_ready": (I, [VP]),
        "scft_batch_create": (I, [P(CSurface), I, P(COptions), P(VP)]),
        "scft_batch_destroy": (I, [VP]),
        "scft_batch_groups": (I, [VP]),
        "scft_batch_locate": (I, [VP, I, P(I), P(I)]),
        "scft_batch_context": (VP, [VP, I]),
        "scft_batch_set_fields": (I, [VP, I, dp]),
        "scft_batch_set_masks": (I, [VP, I, dp]),
        "scft_batch_set_iteration": (I, [VP, I, UL]),
        "scft_batch_set_rng": (I, [VP, I, us3]),
        "scft_batch_set_stop": (I, [VP, I, D]),
        "scft_batch_freeze": (I, [VP, I]),
        "scft_batch_get_fields": (I, [VP, I, dp]),
        "scft_batch_get_densities": (I, [VP, I, dp, dp]),
        "scft_batch_run": (I, [VP, I, I, P(CBatchResult)]),
        "scft_get_fields": (I, [VP, I, dp]),
        "scft_get_densities": (I, [VP, I, dp, dp]),
        "scft_set_fields_all": (I, [VP, dp]),
        "scft_get_fields_all": (I, [VP, dp]),
        "scft_get_densities_all": (I, [VP, dp]),
        "scft_set_fields_all_async": (I, [VP, dp]),
        "scft_get_fields_all_async": (I, [VP, dp]),
        "scft_get_densities_all_async": (I, [VP, dp]),
        "scft_sync": (I, [VP]),
        "scft_propagate": (I, [VP, dp, dp, I, dp]),
        "scft_density": (I, [VP, dp, dp, I, I, I, D, dp]),
        "scft_propagate_static": (I, [VP, dp, dp, I, dp]),
        "scft_static_scratch_bytes": (C.c_size_t, []),
        "scft_enable_timing": (I, [VP, I]),
        "scft_get_timing": (I, [VP, P(CTiming)]),
        "scft_last_error": (C.c_char_p, []),
        "scft_device_memory": (I, [I, P(C.c_size_t), P(C.c_size_t)]),
        "scft_noise_fill": (I, [us3, P(CDerived), dp]),
        "scft_read_counter": (I, [C.c_char_p, P(UL)]),
        "scft_read_restart_fields": (I, [C.c_char_p, P(CDerived), dp]),
        "scft_read_restart_random": (I, [C.c_char_p, us3]),
        "scft_read_mask": (I, [C.c_char_p, P(CDerived), dp]),
        "scft_write_volume_error": (I, [C.c_char_p, D]),
        "scft_write_run_params": (I, [C.c_char_p, P(CSurface), P(CDerived), UL]),
        "scft_write_energies": (I, [C.c_char_p, P(CDerived), P(CIterOut)]),
        "scft_write_snapshot": (I, [C.c_char_p, P(CDerived), UL, dp, dp, us3]),
        "scft_file_names_default": (None, [P(CFileNames)]),
        "scft_set_file_names": (I, [P(CFileNames)]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def exported_symbols():
    """Names of every function include/scft_gpu.h declares."""
    import re
    hdr = (PKG.parent / "include" / "scft_gpu.h").read_text()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(scft_[a-z0-9_]+)\s*\(", hdr)))


class ScftError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = lib().scft_last_error()
        msg = msg.decode() if msg else ""
        super().__init__(f"{where}: {ERRORS.get(code, code)} {msg}")
        self.code = code


def check(code: int, where: str) -> None:
    if code != SCFT_OK:
        raise ScftError(code, where)


__all__ = ["lib", "CSurface", "CDerived", "COptions", "CIterOut", "CTiming", "CBatchResult", "check", "ScftError", "FIELDS",
           "PREC_FP64", "PREC_FP32", "PREC_FP32X2", "exported_symbols"]
