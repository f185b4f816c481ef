"""Generate the golden fixtures in tests/golden/ from the reference solver itself.

Run with SCFT_REFERENCE_DIR naming the reference source tree (the directory
holding SCFT.c); the script stops with an error when it is unset:

    SCFT_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py            # every fixture
    SCFT_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py textnames  # renamed files only

For every case it writes a parameters.h (stimuli-responsive-nanodroplets_gb300.surface)
and the restart-path inputs (counter.dat, restart_fields.dat with %.17g,
restart_random.dat, wMask.dat) into oracle/_ref/golden/<case>/, compiles the
unmodified SCFT.c there (oracle/build.py), runs it and stores its outputs:

* <case>.npz  — full-precision run (every %f/%lf output rewritten to %.17g):
  per-iteration free energy, MF, RMS, chi echo and 17 chemical potentials,
  the last density snapshot (13 phi + 14 w/p columns), the final restart
  fields and RNG state, plus the inputs that produced them.
* text_<case>/ — the same run with the reference's own 6-decimal formats, for
  byte-for-byte checks of the output writers.
* kat_prop_<geom>.npz — funPDESolver called directly in a shared build of the
  reference (main renamed) on seeded q0 and w.

The fixtures are small (grids of a few hundred to a few thousand points, a few
iterations) so the whole set stays well under a few MB.
"""
from __future__ import annotations

import ctypes as C
import importlib
import json
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
srn = importlib.import_module("stimuli-responsive-nanodroplets_gb300")
from oracle import build as obuild  # noqa: E402

GOLD = Path(__file__).resolve().parent
WORK = obuild.REF_OUT / "golden"


def idx_order(nx, ny, nz):
    """idx of each row of a reference grid file (k outer, j, i inner)."""
    out = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                out.append(k + nz * (j + ny * i))
    return np.array(out)


def write_inputs(d: Path, s, w14: np.ndarray, counter: int, seed=(11, 22, 33), mask3=None):
    """The restart-path inputs, under the surface's file names (parameters.h
    COUNTER, RESTART_FIELDS, RESTART_RANDOM, W_MASK)."""
    nx, ny, nz = s.grid()
    order = idx_order(nx, ny, nz)
    (d / s.file_name("COUNTER")).write_text(f"{counter}")
    rows = [" ".join(f"{w14[c, idx]:.17g}" for c in range(14)) + " \n" for idx in order]
    (d / s.file_name("RESTART_FIELDS")).write_text("".join(rows))
    (d / s.file_name("RESTART_RANDOM")).write_text(f"{seed[0]} {seed[1]} {seed[2]}")
    if s.MASK:
        if mask3 is None:
            mask3 = srn.configs.substrate_mask(s)
        rows = [f"{mask3[0, idx]:.17g} {mask3[1, idx]:.17g} {mask3[2, idx]:.17g}\n" for idx in order]
        (d / s.file_name("W_MASK")).write_text("".join(rows))
    return mask3


def parse_grid_file(path: Path, nx, ny, nz, ncols):
    M = nx * ny * nz
    out = np.zeros((ncols, M))
    for line in path.read_text().splitlines():
        v = line.split()
        if not v:
            continue
        i, j, k = int(v[0]), int(v[1]), int(v[2])
        idx = k + nz * (j + ny * i)
        out[:, idx] = [float(x) for x in v[3:3 + ncols]]
    return out


def run_case(name: str, s, w14, counter=1, seed=(11, 22, 33), mask3=None, text=False):
    d = WORK / (name + ("_text" if text else ""))
    if d.exists():
        shutil.rmtree(d)
    d.mkdir(parents=True)
    mask3 = write_inputs(d, s, w14, counter, seed, mask3)
    exe = obuild.build_reference(d, s.to_parameters_h(), full_precision=not text)
    r = subprocess.run([str(exe)], cwd=d, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{name}: reference exited {r.returncode}\n{r.stderr}")
    return d, mask3


def collect(name, s, d: Path, w14, counter, seed, mask3):
    nx, ny, nz = s.grid()
    fe = np.array([[float(x) for x in l.split()] for l in (d / "free_energy.dat").read_text().splitlines() if l.strip()])
    en = np.array([[float(x) for x in l.split()] for l in (d / "energies.dat").read_text().splitlines() if l.strip()])
    dv = np.array([[float(x) for x in l.split()] for l in (d / "deviations.dat").read_text().splitlines() if l.strip()])
    snaps = sorted(d.glob("densities_dbk_*.dat"))
    last = snaps[-1]
    snap = parse_grid_file(last, nx, ny, nz, 27)
    rf = np.loadtxt(d / "restart_fields.dat").reshape(-1, 14)
    order = idx_order(nx, ny, nz)
    restart = np.zeros((14, nx * ny * nz))
    restart[:, order] = rf.T
    rnd = [int(x) for x in (d / "restart_random.dat").read_text().split()]
    np.savez_compressed(
        GOLD / f"{name}.npz",
        surface=json.dumps(s.__dict__), w0=w14, counter=counter, seed0=np.array(seed),
        mask3=mask3 if mask3 is not None else np.zeros((3, nx * ny * nz)),
        free_energy=fe, energies=en, deviations=dv, snap_iter=int(last.stem.split("_")[-1]) - 100000000,
        snap_phi=snap[:13], snap_w=snap[13:], restart_w=restart, restart_rng=np.array(rnd),
        counter_out=int((d / "counter.dat").read_text()), run_txt=(d / "run.txt").read_text())
    print(f"{name}: {len(fe)} iterations, snapshot at {last.name}")


def save_text(name, d: Path, mask_name: str = "wMask.dat"):
    out = GOLD / f"text_{name}"
    if out.exists():
        shutil.rmtree(out)
    out.mkdir()
    for f in sorted(d.iterdir()):
        if f.suffix in (".dat", ".txt", ".error") and f.name != mask_name:
            shutil.copy(f, out / f.name)
    print(f"text_{name}: {sorted(p.name for p in out.iterdir())}")


#: every file-name macro of parameters.h moved off the reference's default
RENAMED = {"COUNTER": "cnt.dat", "DENSITY": "snap_", "DEVIATIONS": "dev.dat", "ENERGY": "en.dat",
           "RESTART_FIELDS": "rf.dat", "RESTART_RANDOM": "rr.dat", "RUN_PARAMS": "params.txt",
           "W_MASK": "mask_in.dat", "FREE_ENERGY": "fe.dat"}


def text_names():
    """The thin-film text case with every file renamed through parameters.h."""
    s = srn.configs.film2d(nx=8, nz=6, ns=16, iters=2)
    s.D_WRT = 1
    s.FILES = dict(RENAMED)
    w = srn.configs.droplet_fields(s, seed=107, radius=0.5)
    d, _ = run_case("textnames", s, w, mask3=srn.configs.substrate_mask(s), text=True)
    np.savez_compressed(GOLD / "text_inputs_names.npz", surface=json.dumps(s.__dict__), w0=w)
    save_text("textnames", d, mask_name=RENAMED["W_MASK"])


# ----------------------------------------------------------------- cases
def case_bulk2d():
    s = srn.configs.bulk2d(nx=32, nz=32, iters=5)
    s.D_WRT = 2
    w = srn.configs.uniform_fields(s.grid(), seed=100, amp=0.1, fields=(0, 1))
    return s, w, None


def case_film2d():
    s = srn.configs.film2d(nx=32, nz=16, ns=64, iters=5)
    s.D_WRT = 5
    w = srn.configs.droplet_fields(s, seed=101, radius=1.2)
    return s, w, srn.configs.substrate_mask(s)


def case_blend3d():
    s = srn.configs.blend3d(n=8, ns=24, seed=7, iters=5)
    s.RELAXATION = 3
    s.D_WRT = 5
    w = srn.configs.uniform_fields(s.grid(), seed=102, amp=0.1, fields=tuple(range(9)))
    return s, w, None


def case_blend3d_full():
    """The four-diblock blend at its full size (64^3, NS 128, noise on) for its
    first six iterations from the bench's start. Only the per-iteration series
    are stored; the test regenerates the start fields from the same seed."""
    s = srn.configs.blend3d(seed=2, iters=6)
    s.D_WRT = 1000
    w = srn.configs.uniform_fields(s.grid(), seed=1000, amp=0.1, fields=tuple(range(9)))
    return s, w


def case_film2d_full():
    """The thin-film droplet configuration at its full size (192x1x96, NS 128,
    MASK 1) for six iterations from a seeded half-disk droplet start."""
    s = srn.configs.film2d(iters=6)
    s.D_WRT = 1000
    w = srn.configs.droplet_fields(s, seed=1000)
    return s, w


def case_bulk2d_full():
    """The 2D bulk melt configuration at its full size (64x1x64, NS 100) for ten
    iterations from a uniform[-0.1, 0.1] start on w_A, w_B."""
    s = srn.configs.bulk2d(iters=10)
    s.D_WRT = 1000
    w = srn.configs.uniform_fields(s.grid(), seed=1000, amp=0.1, fields=(0, 1))
    return s, w


FULL_SERIES = {"blend3d_full": case_blend3d_full, "film2d_full": case_film2d_full, "bulk2d_full": case_bulk2d_full}


def collect_series(name, s, d: Path, w14, counter, seed):
    fe = np.array([[float(x) for x in l.split()] for l in (d / "free_energy.dat").read_text().splitlines() if l.strip()])
    en = np.array([[float(x) for x in l.split()] for l in (d / "energies.dat").read_text().splitlines() if l.strip()])
    dv = np.array([[float(x) for x in l.split()] for l in (d / "deviations.dat").read_text().splitlines() if l.strip()])
    np.savez_compressed(GOLD / f"{name}.npz", surface=json.dumps(s.__dict__), counter=counter, seed0=np.array(seed),
                        w_sum=w14.sum(axis=1), w_sumsq=(w14 * w14).sum(axis=1), free_energy=fe, energies=en,
                        deviations=dv)
    print(f"{name}: {len(fe)} iterations (series only)")


def case_quirks():
    """Even homopolymer contour count (LEN > 1), brush field active with MASK 0,
    energies every 2nd iteration."""
    s = srn.Surface(LX=2.0, LY=1.0, LZ=2.0, ITER=4, D_WRT=3, RELAXATION=0, D_WRT_ENERGIES=2, DT_NOISE=0.5,
                    MASK=0, ENABLE_SEED=0, NS=20, DR_TARGET=0.125, G1=0.1)
    s.VOL_DBK = [0.6, 0.0, 0.0, 0.0]
    s.F_INPUT_DBK = [0.4, 0.5, 0.5, 0.5]
    s.VOL_HOMO = [0.4] + [0.0] * 9
    s.LEN_HOMO = [1.55] + [1.0] * 9
    s.VOL_S = [0.05, 0.0, 0.0]
    s.set_chi("A", "B", 15.0).set_chi("S1", "A", 3.0)
    w = srn.configs.uniform_fields(s.grid(), seed=103, amp=0.2, fields=(0, 1, 10))
    w[13] = np.random.default_rng(104).uniform(-0.05, 0.05, w.shape[1])
    return s, w, None


def case_seed():
    """counter 0: zero fields, drand48 seeded from the clock (MF = 0, so the noise
    never enters), the dbk1 point seed fires in iteration 1."""
    s = srn.configs.film2d(nx=16, nz=16, ns=32, iters=2)
    s.ENABLE_SEED = 1
    s.SEED_STEPS = 1
    s.D_WRT = 1
    w = np.zeros((14, 256))
    return s, w, srn.configs.substrate_mask(s)


def kat_prop(tag: str, s, steps: int, seed: int):
    """funPDESolver on seeded q0, w through a shared build of the reference."""
    d = WORK / f"kat_{tag}"
    if d.exists():
        shutil.rmtree(d)
    so = obuild.build_reference(d, s.to_parameters_h(), full_precision=False, shared=True)
    L = C.CDLL(str(so))
    nx, ny, nz = s.grid()
    M = nx * ny * nz
    N = 2 * (nz + 1) if s.MASK else nz
    for name, val in (("NX", nx), ("NY", ny), ("NZ", nz), ("N", N), ("NS_EFF", steps + 1)):
        C.c_int.in_dll(L, name).value = val
    C.c_ulong.in_dll(L, "iIter").value = 5
    MB = nx * ny * N
    cin = (C.c_double * (2 * MB))()
    cout = (C.c_double * (2 * MB))()
    L.fftw_plan_dft_3d.restype = C.c_void_p
    L.fftw_plan_dft_3d.argtypes = [C.c_int] * 3 + [C.c_void_p] * 2 + [C.c_int, C.c_uint]
    fwd = L.fftw_plan_dft_3d(nx, ny, N, cin, cout, -1, 0)
    bwd = L.fftw_plan_dft_3d(nx, ny, N, cin, cout, 1, 0)
    d_ = srn.derive(s)
    ax, ay, az = d_.c.alphax, d_.c.alphay, d_.c.alphaz
    exparg = np.zeros(MB)
    for i in range(nx):
        for j in range(ny):
            for k in range(N):
                kx = 2.0 * np.pi * (nx / 2.0 - abs(i - nx / 2.0)) / nx
                ky = 2.0 * np.pi * (ny / 2.0 - abs(j - ny / 2.0)) / ny
                kz = 2.0 * np.pi * (N / 2.0 - abs(k - N / 2.0)) / N
                exparg[k + N * (j + ny * i)] = np.exp(-ax * kx * kx - ay * ky * ky - az * kz * kz)
    rng = np.random.default_rng(seed)
    q0 = 1.0 + 0.2 * rng.standard_normal(M)
    w = 0.5 * rng.standard_normal(M)
    qr = np.zeros(M * (steps + 1))
    qr[0::steps + 1] = q0
    dp = C.POINTER(C.c_double)
    L.funPDESolver.argtypes = [C.c_int, C.c_int, dp, dp, dp, C.c_void_p, C.c_void_p, C.c_int]
    L.funPDESolver(0, steps, exparg.ctypes.data_as(dp), qr.ctypes.data_as(dp), w.ctypes.data_as(dp), fwd, bwd, 0)
    q = qr.reshape(M, steps + 1).T.copy()
    np.savez_compressed(GOLD / f"kat_prop_{tag}.npz", surface=json.dumps(s.__dict__), q0=q0, w=w, q=q, exparg=exparg)
    print(f"kat_prop_{tag}: {steps} steps on {nx}x{ny}x{nz}")


def kat_density(tag: str, s, ns: int, blocks, seed: int):
    """funMultiplyQs + funDensity on seeded propagators through a shared build of
    the reference; blocks: (start, stop) pairs of one chain of ns slices."""
    d = WORK / f"kat_{tag}"
    if d.exists():
        shutil.rmtree(d)
    so = obuild.build_reference(d, s.to_parameters_h(), full_precision=False, shared=True)
    L = C.CDLL(str(so))
    nx, ny, nz = s.grid()
    M = nx * ny * nz
    for name, val in (("NX", nx), ("NY", ny), ("NZ", nz), ("NS_EFF", ns)):
        C.c_int.in_dll(L, name).value = val
    rng = np.random.default_rng(seed)
    qf = 1.0 + 0.3 * rng.random((ns, M))
    qb = 1.0 + 0.3 * rng.random((ns, M))
    qr = np.ascontiguousarray(qf.T).reshape(-1)      # AoS: q[s + NS * idx]
    qm = np.ascontiguousarray(qb.T).reshape(-1)
    qc = np.zeros(M * ns)
    dp = C.POINTER(C.c_double)
    L.funMultiplyQs.argtypes = [dp, dp, dp]
    L.funMultiplyQs(qr.ctypes.data_as(dp), qm.ctypes.data_as(dp), qc.ctypes.data_as(dp))
    L.funDensity.argtypes = [C.c_int, C.c_int, dp, dp, C.c_double]
    Q = 1.0 + 0.1 * float(rng.random())
    phis = []
    for start, stop in blocks:
        phi = np.zeros(M)
        L.funDensity(int(start), int(stop), phi.ctypes.data_as(dp), qc.ctypes.data_as(dp), C.c_double(Q))
        phis.append(phi)
    np.savez_compressed(GOLD / f"kat_density_{tag}.npz", grid=np.array([nx, ny, nz]), qf=qf, qb=qb, Q=Q,
                        blocks=np.array(blocks), phi=np.array(phis))
    print(f"kat_density_{tag}: {ns} slices on {nx}x{ny}x{nz}, blocks {blocks}")


def main():
    if not obuild.reference_available():
        raise SystemExit("set SCFT_REFERENCE_DIR to the reference source tree (the directory holding SCFT.c)"
                         if obuild.REFERENCE_DIR is None else f"reference source not found at {obuild.REFERENCE_SRC}")
    if sys.argv[1:] == ["textnames"]:
        text_names()
        return
    if sys.argv[1:] and all(a in FULL_SERIES for a in sys.argv[1:]):
        # full-size series alone (the blend takes about six minutes of one core)
        for name in sys.argv[1:]:
            s, w = FULL_SERIES[name]()
            d, mask3 = run_case(name, s, w)
            collect_series(name, s, d, w, 1, (11, 22, 33))
            shutil.rmtree(d)  # the run folder holds full-size text files
        return
    for name, fn in (("bulk2d", case_bulk2d), ("film2d", case_film2d), ("blend3d", case_blend3d),
                     ("quirks", case_quirks)):
        s, w, mask3 = fn()
        d, mask3 = run_case(name, s, w, mask3=mask3)
        collect(name, s, d, w, 1, (11, 22, 33), mask3)
    # counter-0 start with the point seed
    s, w, mask3 = case_seed()
    d, mask3 = run_case("seed", s, w, counter=0, mask3=mask3)
    collect("seed", s, d, w, 0, (0, 0, 0), mask3)
    # native-format text of a small run, for byte-exact writer checks
    s = srn.configs.bulk2d(nx=12, nz=10, iters=3)
    s.D_WRT = 2
    w = srn.configs.uniform_fields(s.grid(), seed=105, amp=0.1, fields=(0, 1))
    d, _ = run_case("textcase", s, w, text=True)
    np.savez_compressed(GOLD / "text_inputs.npz", surface=json.dumps(s.__dict__), w0=w)
    save_text("textcase", d)
    s2 = srn.configs.film2d(nx=8, nz=6, ns=16, iters=1)
    s2.D_WRT = 1
    w2 = srn.configs.droplet_fields(s2, seed=106, radius=0.5)
    d2, _ = run_case("textfilm", s2, w2, mask3=srn.configs.substrate_mask(s2), text=True)
    np.savez_compressed(GOLD / "text_inputs_film.npz", surface=json.dumps(s2.__dict__), w0=w2)
    save_text("textfilm", d2)
    text_names()
    # volume check failure
    s3 = srn.configs.bulk2d(nx=8, nz=8, iters=1)
    s3.VOL_DBK = [0.9, 0.0, 0.0, 0.0]
    d3 = WORK / "volfail_text"
    if d3.exists():
        shutil.rmtree(d3)
    d3.mkdir(parents=True)
    exe = obuild.build_reference(d3, s3.to_parameters_h(), full_precision=False)
    subprocess.run([str(exe)], cwd=d3, capture_output=True)
    save_text("volfail", d3)
    # per-function propagator checks
    kat_prop("periodic2d", srn.configs.bulk2d(nx=32, nz=24, iters=1), steps=12, seed=201)
    kat_prop("dirichlet2d", srn.configs.film2d(nx=24, nz=16, ns=64, iters=1), steps=12, seed=202)
    kat_prop("periodic3d", srn.configs.blend3d(n=8, ns=24, iters=1), steps=6, seed=203)
    # odd interval count (the dropped point stop-1), an even one, and a block starting mid-chain
    kat_density("2d", srn.configs.bulk2d(nx=16, nz=12, iters=1), ns=21, blocks=[(0, 20), (0, 9), (9, 20), (3, 14)],
                seed=204)


if __name__ == "__main__":
    main()
