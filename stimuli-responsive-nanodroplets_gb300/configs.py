"""Named workloads and their seeded synthetic inputs.

The reference ships no benchmark inputs and no initial-state generator beyond a
zero start with a point seed (SCFT.c:799-842, :2346-2361); these generators make
the restart-path inputs (fields, grafting masks, RNG state) of each workload
from a seed, with the shapes and value ranges the workloads name.
"""
from __future__ import annotations

import numpy as np

from .surface import Surface


# ------------------------------------------------------------------ surfaces
def bulk2d(nx: int = 64, nz: int = 64, iters: int = 2000) -> Surface:
    """Symmetric AB diblock melt, bulk (MASK 0): chi_AB N = 20, NS = 100, G1 = 0.1,
    noise off; 64x1x64 at the default size (DR_TARGET = 0.125)."""
    s = Surface(LX=nx * 0.125, LY=1.0, LZ=nz * 0.125, ITER=iters, D_WRT=iters, RELAXATION=0, D_WRT_ENERGIES=1,
                DT_NOISE=0.0, MASK=0, ENABLE_SEED=0, NS=100, DR_TARGET=0.125, G1=0.1)
    s.VOL_DBK = [1.0, 0.0, 0.0, 0.0]
    s.F_INPUT_DBK = [0.5, 0.5, 0.5, 0.5]
    s.set_chi("A", "B", 20.0)
    return s


def film2d(nx: int = 192, nz: int = 96, ns: int = 128, chi_ab: float = 20.0, chi_ac: float = 40.0,
           iters: int = 5000) -> Surface:
    """Thin-film nanodroplet (MASK 1): AB diblock f = 0.5 at VOL 0.20, homopolymer C
    solvent at 0.80, brush S1 (VOL 0.05, LEN 0.5) grafted at z = 0; chi_AB N = 20,
    chi_AC N = 40, chi_BC N = 35, chi_S1C N = 5, chi_S1A N = chi_S1B N = 10;
    LX = 24, LZ = 12 (192x1x96 at DR_TARGET 0.125), NS = 128, G1 = 0.05."""
    s = Surface(LX=nx * 0.125, LY=1.0, LZ=nz * 0.125, ITER=iters, D_WRT=iters, RELAXATION=0, D_WRT_ENERGIES=1,
                DT_NOISE=0.0, MASK=1, ENABLE_SEED=0, NS=ns, DR_TARGET=0.125, G1=0.05)
    s.VOL_DBK = [0.20, 0.0, 0.0, 0.0]
    s.F_INPUT_DBK = [0.5, 0.5, 0.5, 0.5]
    s.VOL_HOMO = [0.0, 0.0, 0.80] + [0.0] * 7
    s.VOL_S = [0.05, 0.0, 0.0]
    s.LEN_S = [0.5, 0.1, 0.1]
    s.set_chi("A", "B", chi_ab).set_chi("A", "C", chi_ac).set_chi("B", "C", 35.0)
    s.set_chi("S1", "C", 5.0).set_chi("S1", "A", 10.0).set_chi("S1", "B", 10.0)
    return s


def blend3d(n: int = 64, ns: int = 128, seed: int = 2, iters: int = 3000) -> Surface:
    """3D bulk blend: 4 diblocks (f = .3 .5 .5 .7, LEN 1 1 .5 1.5, VOL .2 each) plus
    homopolymers A, B, C (VOL .1 .05 .05, LEN .5 .5 1); symmetric chi N matrix
    drawn uniform in [5, 40] from the seed; LX = LY = LZ = 10 (64^3), NS = 128,
    G1 = 0.1, RELAXATION = 500 with noise amplitude 0.1."""
    L = 10.0 * n / 64
    s = Surface(LX=L, LY=L, LZ=L, ITER=iters, D_WRT=iters, RELAXATION=500, D_WRT_ENERGIES=1, DT_NOISE=0.1, MASK=0,
                ENABLE_SEED=0, NS=ns, DR_TARGET=10.0 / 64, G1=0.1)
    s.VOL_DBK = [0.2, 0.2, 0.2, 0.2]
    s.F_INPUT_DBK = [0.3, 0.5, 0.5, 0.7]
    s.LEN_DBK = [1.0, 1.0, 0.5, 1.5]
    s.VOL_HOMO = [0.1, 0.05, 0.05] + [0.0] * 7
    s.LEN_HOMO = [0.5, 0.5, 1.0] + [1.0] * 7
    rng = np.random.default_rng(seed)
    for f in range(10):
        for g in range(f + 1, 10):
            s.set_chi(f, g, float(rng.uniform(5.0, 40.0)))
    return s


# -------------------------------------------------------------- input fields
def idx_coords(nx: int, ny: int, nz: int):
    """(i, j, k) of every idx = k + NZ*(j + NY*i) (SCFT.c:773)."""
    idx = np.arange(nx * ny * nz)
    return idx // (ny * nz), (idx // nz) % ny, idx % nz


def uniform_fields(shape, seed: int, amp: float, fields=(0, 1)) -> np.ndarray:
    """w14 with the given fields i.i.d. uniform in [-amp, amp], everything else 0."""
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    w = np.zeros((14, nx * ny * nz))
    for f in fields:
        w[f] = rng.uniform(-amp, amp, nx * ny * nz)
    return w


def droplet_fields(s: Surface, seed: int, radius: float = 6.0, strength: float = 4.0, amp: float = 0.05) -> np.ndarray:
    """Half-disk droplet of disordered AB on the substrate (z = 0) in C solvent.

    Inside the half disk of the given radius (R_g units, centred at LX/2 on the
    wall) the solvent field w_C is raised, outside the copolymer fields w_A and
    w_B are raised; every field also gets uniform[-amp, amp] noise."""
    nx, ny, nz = s.grid()
    i, j, k = idx_coords(nx, ny, nz)
    dx, dz = s.LX / nx, s.LZ / nz
    x = (i + 0.5) * dx - s.LX / 2.0
    z = (k + 1) * dz  # the Dirichlet wall sits one spacing below k = 0
    inside = (x * x + z * z) < radius * radius
    rng = np.random.default_rng(seed)
    w = np.zeros((14, nx * ny * nz))
    w[0] = np.where(inside, 0.0, strength)
    w[1] = np.where(inside, 0.0, strength)
    w[2] = np.where(inside, strength, 0.0)
    for f in (0, 1, 2, 10):
        w[f] += rng.uniform(-amp, amp, nx * ny * nz)
    return w


def substrate_mask(s: Surface, layer: int = 0) -> np.ndarray:
    """wMask columns: S1 grafted (1) on the k = layer plane, S2 and S3 empty."""
    nx, ny, nz = s.grid()
    _, _, k = idx_coords(nx, ny, nz)
    m = np.zeros((3, nx * ny * nz))
    m[0] = (k == layer).astype(float)
    return m


def sweep_surfaces(n: int = 16, seed: int = 3, sizes=((64, 64), (96, 64), (128, 96), (192, 96), (192, 128)),
                   ns_range=(64, 128)):
    """The 2D droplet sweep: chi_AB N x chi_AC N on an n x n grid over [10,30]x[20,60],
    film2d chemistry, grid size and NS drawn per point from the seed."""
    rng = np.random.default_rng(seed)
    out = []
    for a in range(n):
        for c in range(n):
            chi_ab = 10.0 + 20.0 * a / max(n - 1, 1)
            chi_ac = 20.0 + 40.0 * c / max(n - 1, 1)
            nx, nz = sizes[int(rng.integers(len(sizes)))]
            ns = int(rng.integers(ns_range[0], ns_range[1] + 1))
            out.append(film2d(nx=nx, nz=nz, ns=ns, chi_ab=chi_ab, chi_ac=chi_ac))
    return out


# ------------------------------------------------------- phase-diagram planes
# The phase diagram is a (chi_AB N, chi_AC N) grid repeated over three planes,
# one per starting contact angle; a plane fixes the other interactions. Here a
# plane sets the brush-S1 interactions of the thin film (S1 neutral, S1
# solvent-philic, S1 copolymer-philic) and chi_BC N of the 3D bulk blend.
PLANES = (
    {"name": "P0", "S1C": 5.0, "S1AB": 10.0, "BC": 35.0},   # near 90 degrees
    {"name": "P1", "S1C": 0.0, "S1AB": 20.0, "BC": 25.0},   # near dewetted
    {"name": "P2", "S1C": 20.0, "S1AB": 0.0, "BC": 45.0},   # near wetted
)


def chi_axes(n: int = 24, ab=(10.0, 30.0), ac=(20.0, 60.0)):
    """The (chi_AB N, chi_AC N) grid values of an n x n plane."""
    return (np.array([ab[0] + (ab[1] - ab[0]) * i / max(n - 1, 1) for i in range(n)]),
            np.array([ac[0] + (ac[1] - ac[0]) * j / max(n - 1, 1) for j in range(n)]))


def film_point(chi_ab: float, chi_ac: float, plane: dict, nx: int = 192, nz: int = 96, ns: int = 100) -> Surface:
    """Thin-film droplet chemistry at one phase-diagram point of a plane."""
    s = film2d(nx=nx, nz=nz, ns=ns, chi_ab=chi_ab, chi_ac=chi_ac)
    s.set_chi("S1", "C", plane["S1C"]).set_chi("S1", "A", plane["S1AB"]).set_chi("S1", "B", plane["S1AB"])
    return s


def bulk3d_point(chi_ab: float, chi_ac: float, plane: dict, n: int = 64, ns: int = 100) -> Surface:
    """3D bulk (MASK 0) AB diblock f = 0.5 at VOL 0.4 in homopolymer C solvent at
    0.6; LX = LY = LZ = 8 R_g (64^3 at DR_TARGET 0.125), G1 = 0.05, noise off."""
    L = n * 0.125
    s = Surface(LX=L, LY=L, LZ=L, ITER=5000, D_WRT=5000, RELAXATION=0, D_WRT_ENERGIES=1, DT_NOISE=0.0, MASK=0,
                ENABLE_SEED=0, NS=ns, DR_TARGET=0.125, G1=0.05)
    s.VOL_DBK = [0.4, 0.0, 0.0, 0.0]
    s.F_INPUT_DBK = [0.5, 0.5, 0.5, 0.5]
    s.VOL_HOMO = [0.0, 0.0, 0.6] + [0.0] * 7
    s.set_chi("A", "B", chi_ab).set_chi("A", "C", chi_ac).set_chi("B", "C", plane["BC"])
    return s


def seed_fields(s: Surface, kind: str, seed: int, amp: float = 0.05) -> np.ndarray:
    """Synthetic first-pass seeds: "lamellar" (w_A - w_B ~ cos along x),
    "cylinder" (cos along x times cos along z), "disordered" (noise only), inside
    the droplet of a film (MASK 1) or everywhere in a bulk box; every field gets
    uniform[-amp, amp] noise from the seed."""
    nx, ny, nz = s.grid()
    i, j, k = idx_coords(nx, ny, nz)
    if s.MASK:
        w = droplet_fields(s, seed=seed, radius=min(6.0, 0.3 * s.LX, 0.6 * s.LZ), amp=amp)
    else:
        w = uniform_fields((nx, ny, nz), seed=seed, amp=amp, fields=(0, 1, 2))
    periods = 4.0
    if kind == "lamellar":
        pat = np.cos(2.0 * np.pi * periods * i / nx)
    elif kind == "cylinder":
        pat = np.cos(2.0 * np.pi * periods * i / nx) * np.cos(2.0 * np.pi * 2.0 * k / nz)
    elif kind == "disordered":
        pat = np.zeros(nx * ny * nz)
    else:
        raise ValueError(f"unknown seed kind {kind!r}")
    w[0] += 1.5 * pat
    w[1] -= 1.5 * pat
    return w
