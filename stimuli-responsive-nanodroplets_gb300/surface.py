"""The ``parameters.h`` run surface of SCFT.c as a Python value.

SCFT.c takes every run parameter as a compile-time macro from ``parameters.h``
(parameters.h:1-190, included at SCFT.c:10). :class:`Surface` holds the same
macros, writes a ``parameters.h`` that the reference solver and this package's
C host both compile against, and parses such a header back. It replaces the
generator script that parameters.h:159 mentions but the reference does not ship.

Field order everywhere in this package is the reference's 13-field order
(getCHI_N_EFF table, SCFT.c:1930-1945): A B C D E F G H I J S1 S2 S3.
"""
from __future__ import annotations

import dataclasses
import re
from typing import Dict, List

FIELDS: List[str] = ["A", "B", "C", "D", "E", "F", "G", "H", "I", "J", "S1", "S2", "S3"]
HOMO = FIELDS[:10]


def chi_macro(f: int, g: int) -> str:
    """Macro name parameters.h uses for the chi*N of fields f and g (f != g).

    A-J pairs are CHI_N_XY with X before Y (parameters.h:22-74); brush pairs are
    CHI_N_Sa_Sb (parameters.h:124-126) and brush/free pairs CHI_N_Sa_X
    (parameters.h:128-157).
    """
    if f == g:
        raise ValueError("no self interaction macro")
    a, b = sorted((f, g))
    if b < 10:
        return f"CHI_N_{FIELDS[a]}{FIELDS[b]}"
    if a >= 10:
        return f"CHI_N_{FIELDS[a]}_{FIELDS[b]}"
    return f"CHI_N_{FIELDS[b]}_{FIELDS[a]}"


INT_MACROS = ["ITER", "D_WRT", "RELAXATION", "D_WRT_ENERGIES", "MASK", "ENABLE_SEED", "SEED_STEPS",
              "SEED_AREA_DELTA", "NS"]


#: the file-name macros of parameters.h (parameters.h:181-190) and the reference's names
FILE_MACROS: Dict[str, str] = {
    "COUNTER": "counter.dat", "DENSITY": "densities_dbk_", "DEVIATIONS": "deviations.dat",
    "ENERGY": "energies.dat", "RESTART_FIELDS": "restart_fields.dat", "RESTART_RANDOM": "restart_random.dat",
    "RUN_PARAMS": "run.txt", "W_MASK": "wMask.dat", "FREE_ENERGY": "free_energy.dat",
}


def _chi_names() -> List[str]:
    names = []
    for f in range(10):
        for g in range(f + 1, 10):
            names.append(chi_macro(f, g))
    return names


@dataclasses.dataclass
class Surface:
    """All macros of parameters.h, with the reference's meaning (README.md:14-33)."""

    LX: float = 8.0
    LY: float = 1.0
    LZ: float = 8.0
    ITER: int = 2000
    D_WRT: int = 1000
    RELAXATION: int = 0
    D_WRT_ENERGIES: int = 1
    DT_NOISE: float = 0.0
    MASK: int = 0
    ENABLE_SEED: int = 0
    SEED_STEPS: int = 1
    SEED_AREA_DELTA: int = 1
    NS: int = 100
    DR_TARGET: float = 0.125
    G1: float = 0.1
    chi: Dict[str, float] = dataclasses.field(default_factory=dict)
    F_INPUT_DBK: List[float] = dataclasses.field(default_factory=lambda: [0.5, 0.5, 0.5, 0.5])
    LEN_DBK: List[float] = dataclasses.field(default_factory=lambda: [1.0, 1.0, 1.0, 1.0])
    VOL_DBK: List[float] = dataclasses.field(default_factory=lambda: [0.0, 0.0, 0.0, 0.0])
    VOL_HOMO: List[float] = dataclasses.field(default_factory=lambda: [0.0] * 10)
    LEN_HOMO: List[float] = dataclasses.field(default_factory=lambda: [1.0] * 10)
    VOL_S: List[float] = dataclasses.field(default_factory=lambda: [0.0, 0.0, 0.0])
    LEN_S: List[float] = dataclasses.field(default_factory=lambda: [0.1, 0.1, 0.1])
    #: file names (macro -> name); missing macros keep the reference's names
    FILES: Dict[str, str] = dataclasses.field(default_factory=dict)

    def file_name(self, macro: str) -> str:
        return (getattr(self, "FILES", None) or {}).get(macro, FILE_MACROS[macro])

    # ------------------------------------------------------------------ chi
    def chi_n(self, f: int, g: int) -> float:
        if f == g:
            return 0.0
        return float(self.chi.get(chi_macro(f, g), 0.0))

    def set_chi(self, f, g, value: float) -> "Surface":
        fi = FIELDS.index(f) if isinstance(f, str) else int(f)
        gi = FIELDS.index(g) if isinstance(g, str) else int(g)
        self.chi[chi_macro(fi, gi)] = float(value)
        return self

    def chi_table(self) -> List[List[float]]:
        return [[self.chi_n(f, g) for g in range(13)] for f in range(13)]

    # -------------------------------------------------------------- writing
    def to_parameters_h(self) -> str:
        """Return a parameters.h with the reference's macro set (parameters.h:1-190)."""

        def num(v) -> str:
            r = repr(float(v))
            return r if ("." in r or "e" in r or "inf" in r or "nan" in r) else r + ".0"

        L = ["// Generated run surface for SCFT.c (same macros as the reference parameters.h)"]
        L += [f"#define LX {num(self.LX)}", f"#define LY {num(self.LY)}", f"#define LZ {num(self.LZ)}", ""]
        L += [f"#define ITER {int(self.ITER)}", f"#define D_WRT {int(self.D_WRT)}",
              f"#define RELAXATION {int(self.RELAXATION)}", f"#define D_WRT_ENERGIES {int(self.D_WRT_ENERGIES)}",
              f"#define DT_NOISE {num(self.DT_NOISE)}", f"#define MASK {int(self.MASK)}", ""]
        L += [f"#define ENABLE_SEED {int(self.ENABLE_SEED)}", f"#define SEED_STEPS {int(self.SEED_STEPS)}",
              f"#define SEED_AREA_DELTA {int(self.SEED_AREA_DELTA)}", ""]
        L += [f"#define NS {int(self.NS)}", f"#define DR_TARGET {num(self.DR_TARGET)}",
              "#define DS (1.0 / (NS - 1))", f"#define G1 {num(self.G1)}", ""]
        for f in range(10):
            for g in range(f + 1, 10):
                L.append(f"#define {chi_macro(f, g)} {num(self.chi_n(f, g))}")
        L.append("")
        for d in range(4):
            L.append(f"#define F_INPUT_DBK_{d + 1} {num(self.F_INPUT_DBK[d])}")
            L.append(f"#define LEN_DBK_{d + 1} {num(self.LEN_DBK[d])}")
        for d in range(4):
            L.append(f"#define VOL_DBK_{d + 1} {num(self.VOL_DBK[d])}")
        for h in range(10):
            L.append(f"#define VOL_HOMOPOLYMER_{HOMO[h]} {num(self.VOL_HOMO[h])}")
        for h in range(10):
            L.append(f"#define LEN_HOMO_{HOMO[h]} {num(self.LEN_HOMO[h])}")
        L.append("")
        for s in range(3):
            L.append(f"#define VOL_S{s + 1} {num(self.VOL_S[s])}")
            L.append(f"#define LEN_S{s + 1} {num(self.LEN_S[s])}")
        L.append("")
        for a, b in ((10, 11), (10, 12), (11, 12)):
            L.append(f"#define {chi_macro(a, b)} {num(self.chi_n(a, b))}")
        for s in range(10, 13):
            for f in range(10):
                L.append(f"#define {chi_macro(s, f)} {num(self.chi_n(s, f))}")
        L.append("")
        for gi in range(2, 14):
            L.append(f"#define G{gi}   G1 / 6.0")
        L += ["", "#define DX  (LX/NX)", "#define DY  (LY/NY)", "#define DZ  (LZ/NZ)", "",
              "#define ALPHAX  (DS/(DX*DX))", "#define ALPHAY  (DS/(DY*DY))", "#define ALPHAZ  (DS/(DZ*DZ))", "",
              "// File names"]
        L += [f'#define {m} "{self.file_name(m)}"' for m in FILE_MACROS]
        L.append("")
        return "\n".join(L)

    # -------------------------------------------------------------- parsing
    @classmethod
    def from_parameters_h(cls, text: str) -> "Surface":
        """Parse the numeric macros of a parameters.h (comments allowed)."""
        vals: Dict[str, float] = {}
        files: Dict[str, str] = {}
        for line in text.splitlines():
            line = line.split("//", 1)[0]
            m = re.match(r"\s*#define\s+([A-Z0-9_]+)\s+(.+?)\s*$", line)
            if not m:
                continue
            name, expr = m.group(1), m.group(2)
            q = re.fullmatch(r'"([^"]*)"', expr)
            if q and name in FILE_MACROS:
                files[name] = q.group(1)
                continue
            try:
                vals[name] = float(expr)
            except ValueError:
                continue  # derived macros (DS, G2.., DX..)
        s = cls()
        s.FILES = {k: v for k, v in files.items() if v != FILE_MACROS[k]}
        for name in ["LX", "LY", "LZ", "DT_NOISE", "DR_TARGET", "G1"]:
            if name in vals:
                setattr(s, name, vals[name])
        for name in INT_MACROS:
            if name in vals:
                setattr(s, name, int(vals[name]))
        for f in range(13):
            for g in range(f + 1, 13):
                key = chi_macro(f, g)
                if key in vals:
                    s.chi[key] = vals[key]
        for d in range(4):
            s.F_INPUT_DBK[d] = vals.get(f"F_INPUT_DBK_{d + 1}", s.F_INPUT_DBK[d])
            s.LEN_DBK[d] = vals.get(f"LEN_DBK_{d + 1}", s.LEN_DBK[d])
            s.VOL_DBK[d] = vals.get(f"VOL_DBK_{d + 1}", s.VOL_DBK[d])
        for h in range(10):
            s.VOL_HOMO[h] = vals.get(f"VOL_HOMOPOLYMER_{HOMO[h]}", s.VOL_HOMO[h])
            s.LEN_HOMO[h] = vals.get(f"LEN_HOMO_{HOMO[h]}", s.LEN_HOMO[h])
        for k in range(3):
            s.VOL_S[k] = vals.get(f"VOL_S{k + 1}", s.VOL_S[k])
            s.LEN_S[k] = vals.get(f"LEN_S{k + 1}", s.LEN_S[k])
        return s

    def copy(self) -> "Surface":
        return dataclasses.replace(self, chi=dict(self.chi), F_INPUT_DBK=list(self.F_INPUT_DBK),
                                   LEN_DBK=list(self.LEN_DBK), VOL_DBK=list(self.VOL_DBK),
                                   VOL_HOMO=list(self.VOL_HOMO), LEN_HOMO=list(self.LEN_HOMO),
                                   VOL_S=list(self.VOL_S), LEN_S=list(self.LEN_S),
                                   FILES=dict(getattr(self, "FILES", None) or {}))

    def grid(self):
        """(NX, NY, NZ) by the reference's rounding rule (SCFT.c:103-105)."""

        def n(L):
            return 1 if L == 1.0 else int((L / self.DR_TARGET) + 0.5)

        return n(self.LX), n(self.LY), n(self.LZ)
