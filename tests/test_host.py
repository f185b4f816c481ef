"""Host side of the library, no GPU: exported symbols, parameter derivation,
the reference's text formats byte for byte, the drand48 noise replay, readers.
"""
import ctypes as C
import importlib
import json
import os

import numpy as np
import pytest

from conftest import GOLD, load_golden, surface_from_json

CASES = ["bulk2d", "film2d", "blend3d", "quirks", "seed"]


def test_library_exports_every_header_symbol(srn):
    L = importlib.import_module("stimuli-responsive-nanodroplets_gb300._lib")
    lib = L.lib()
    names = L.exported_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_layouts_match_header(tmp_path):
    """Every public struct of include/scft_gpu.h has the size and field offsets
    that the ctypes mirror in _lib.py assumes (a C program built against the
    header prints them)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    L = importlib.import_module("stimuli-responsive-nanodroplets_gb300._lib")
    structs = {"scft_surface": L.CSurface, "scft_derived": L.CDerived, "scft_options": L.COptions,
               "scft_iter_out": L.CIterOut, "scft_batch_result": L.CBatchResult, "scft_timing": L.CTiming}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "scft_gpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            parts = line.split()
            got[(parts[0], parts[1])] = int(parts[2])
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


@pytest.mark.parametrize("case", CASES)
def test_derive_matches_oracle(case, srn, golden, oracle_mod):
    g = golden(case)
    S = g["S"]
    d = srn.derive(S)
    o = oracle_mod.Oracle(S).derived()
    assert tuple(d.grid) == o["grid"]
    assert d.c.n_active == o["n_active"]
    assert list(d.active) == list(o["active"])
    lens = list(d.ns_dbk) + list(d.ns_homo) + list(d.ns_s)
    assert lens == list(o["len"])
    assert list(d.ns_dbk_x) == list(o["nsx"][:4]) and list(d.ns_dbk_y) == list(o["nsy"][:4])
    assert d.c.ds == o["ds"]
    assert [d.c.alphax, d.c.alphay, d.c.alphaz] == list(o["alpha"])
    assert d.c.coating_vol == o["coating"]
    assert list(d.phi_avg) == list(o["phi_avg"])
    assert np.array_equal(d.chi_eff, o["chi"])
    alphas = list(d.alpha_dbk) + list(d.alpha_homo) + list(d.alpha_s)
    assert alphas == list(o["alpha_sp"])


def test_derive_even_homopolymer_count(srn):
    """LEN > 1 can leave an even contour count (the '> NS' branch, SCFT.c:173)."""
    s = srn.Surface(NS=20)
    s.VOL_HOMO = [1.0] + [0.0] * 9
    s.LEN_HOMO = [1.55] + [1.0] * 9
    d = srn.derive(s)
    assert int(d.ns_homo[0]) == 30


def test_volume_check(srn, tmp_path):
    s = srn.configs.bulk2d(nx=8, nz=8, iters=1)
    s.VOL_DBK = [0.9, 0.0, 0.0, 0.0]
    d = srn.derive(s)
    assert d.status == -5 and not d.c.volume_ok
    srn.write_volume_error(tmp_path, d.c.volume_sum)
    want = (GOLD / "text_volfail" / "DENSITY_CHECK_FAIL.error").read_bytes()
    assert (tmp_path / "DENSITY_CHECK_FAIL.error").read_bytes() == want


def test_parameters_h_roundtrip(srn):
    for s in (srn.configs.film2d(), srn.configs.blend3d(), srn.configs.bulk2d()):
        t = s.to_parameters_h()
        s2 = srn.Surface.from_parameters_h(t)
        assert s2.to_parameters_h() == t
        assert s2.chi_table() == s.chi_table()


def _libc_gauss(state):
    """Marsaglia polar draws with libc's erand48 (the generator drand48 uses)."""
    libc = C.CDLL(None)
    libc.erand48.restype = C.c_double
    libc.erand48.argtypes = [C.POINTER(C.c_ushort)]
    while True:
        x1 = 2.0 * libc.erand48(state) - 1.0
        x2 = 2.0 * libc.erand48(state) - 1.0
        w = x1 * x1 + x2 * x2
        if w < 1.0:
            break
    return x1 * np.sqrt((-2.0 * np.log(w)) / w)


def test_noise_fill_replays_drand48(srn):
    s = srn.configs.blend3d(n=4, ns=24, iters=1)
    d = srn.derive(s)
    seed = (123, 456, 789)
    noise, st = srn.noise_fill(seed, d)
    ref_state = (C.c_ushort * 3)(*seed)
    nx, ny, nz = d.grid
    na = d.c.n_active
    ref = np.empty_like(noise)
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                idx = k + nz * (j + ny * i)
                for a in range(na):
                    ref[a, idx] = _libc_gauss(ref_state)
    assert st == tuple(ref_state)
    np.testing.assert_allclose(noise, ref, rtol=1e-15, atol=0)


def _oracle_run_text(srn, oracle_mod, surface, w0, mask3):
    """Run the oracle through a text case and write every output with the
    library's writers, as the reference would at these iterations."""
    o = oracle_mod.Oracle(surface)
    o.set_fields(w0)
    if mask3 is not None:
        o.set_masks(mask3)
    o.set_iter(1)
    o.set_rng((11, 22, 33))
    return o


@pytest.mark.parametrize("name,inputs,mask", [("textcase", "text_inputs", False), ("textfilm", "text_inputs_film", True),
                                               ("textnames", "text_inputs_names", True)])
def test_writers_byte_exact(name, inputs, mask, srn, oracle_mod, tmp_path):
    """The library's writers against SCFT.c's files; textnames renames every
    file through the file-name macros of parameters.h."""
    gi = dict(np.load(GOLD / f"{inputs}.npz"))
    S = surface_from_json(srn, gi["surface"])
    d = srn.derive(S)
    m3 = srn.configs.substrate_mask(S) if mask else None
    o = _oracle_run_text(srn, oracle_mod, S, gi["w0"], m3)
    saved = (11, 22, 33)
    srn.set_file_names(S)
    try:
        for _ in range(int(S.ITER)):
            r = o.iterate(1)[0]
            it = int(r[0])
            rec = srn.IterOut(it, r[1], r[2], r[3], r[4:21], r[21:38], 0)
            if it % int(S.D_WRT_ENERGIES) == 0:
                srn.write_energies(tmp_path, d, rec)
            if it % int(S.D_WRT) == 0 or it == 1:
                phi, _ = o.densities()
                srn.write_snapshot(tmp_path, d, it, phi, o.get_fields(), saved)
                saved = o.get_rng()
        srn.write_run_params(tmp_path, S, d, 1)
    finally:
        srn.set_file_names(None)
    ref_dir = GOLD / f"text_{name}"
    for f in sorted(os.listdir(ref_dir)):
        got = (tmp_path / f).read_bytes()
        want = (ref_dir / f).read_bytes()
        assert got == want, f


def test_readers_roundtrip(srn, tmp_path):
    s = srn.configs.film2d(nx=8, nz=6, ns=16, iters=1)
    d = srn.derive(s)
    M = d.M
    rng = np.random.default_rng(0)
    w = np.round(rng.uniform(-1, 1, (14, M)), 6)
    phi = np.round(rng.uniform(0, 1, (13, M)), 6)
    srn.write_snapshot(tmp_path, d, 7, phi, w, (1, 2, 3))
    assert srn.read_counter(tmp_path) == 7
    np.testing.assert_allclose(srn.read_restart_fields(tmp_path, d), w, atol=5e-7)
    assert srn.read_restart_random(tmp_path) == (1, 2, 3)
    m = srn.configs.substrate_mask(s)
    i, j, k = srn.configs.idx_coords(*d.grid)
    rows = []
    for kk in range(d.grid[2]):
        for jj in range(d.grid[1]):
            for ii in range(d.grid[0]):
                idx = kk + d.grid[2] * (jj + d.grid[1] * ii)
                rows.append(f"{m[0, idx]} {m[1, idx]} {m[2, idx]}\n")
    (tmp_path / "wMask.dat").write_text("".join(rows))
    np.testing.assert_array_equal(srn.read_mask(tmp_path, d), m)


def test_allocation_free_entry_point_names_no_allocator():
    """scft_propagate_static's source calls no device or pinned allocator (its
    working buffers are the file-scope array)."""
    import re
    src = (GOLD.parents[1] / "stimuli-responsive-nanodroplets_gb300" / "csrc" / "scft_noalloc.cu").read_text()
    code = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    code = re.sub(r"//[^\n]*", "", code)
    for name in ("cudaMalloc", "cudaFree", "cudaMallocAsync", "cudaFreeAsync", "cudaMallocHost", "cudaHostAlloc",
                 "cudaMallocManaged", "malloc(", "new "):
        assert name not in code, name


def test_file_name_macros_round_trip(srn):
    """parameters.h's file-name macros survive the header generator and parser;
    a header with the reference's names keeps no overrides."""
    s = srn.configs.film2d(nx=8, nz=6, ns=16, iters=1)
    assert srn.Surface.from_parameters_h(s.to_parameters_h()).FILES == {}
    s.FILES = {"COUNTER": "runs/cnt.dat", "DENSITY": "snap_", "W_MASK": "m.dat"}
    back = srn.Surface.from_parameters_h(s.to_parameters_h())
    assert back.FILES == s.FILES
    assert back.file_name("ENERGY") == "energies.dat" and back.file_name("COUNTER") == "runs/cnt.dat"

