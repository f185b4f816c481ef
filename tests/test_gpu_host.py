"""The drop-in C host (csrc/scft_main.c) on the GPU: run in a directory laid out
like the reference's, it must write the same files, byte for byte, as SCFT.c
wrote for the same inputs (tests/golden/text_*)."""
import importlib
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLD, surface_from_json

pytestmark = pytest.mark.gpu


def write_inputs(srn, d, S, w14, path, mask3):
    nx, ny, nz = S.grid()
    rows = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                idx = k + nz * (j + ny * i)
                rows.append(" ".join(f"{w14[c, idx]:.17g}" for c in range(14)) + " \n")
    (path / S.file_name("RESTART_FIELDS")).write_text("".join(rows))
    (path / S.file_name("COUNTER")).write_text("1")
    (path / S.file_name("RESTART_RANDOM")).write_text("11 22 33")
    if mask3 is not None:
        mrows = []
        for k in range(nz):
            for j in range(ny):
                for i in range(nx):
                    idx = k + nz * (j + ny * i)
                    mrows.append(f"{mask3[0, idx]:.17g} {mask3[1, idx]:.17g} {mask3[2, idx]:.17g}\n")
        (path / S.file_name("W_MASK")).write_text("".join(mrows))


@pytest.mark.parametrize("name,inputs,mask", [("textcase", "text_inputs", False), ("textfilm", "text_inputs_film", True),
                                               ("textnames", "text_inputs_names", True)])
def test_c_host_writes_reference_files(name, inputs, mask, srn, tmp_path):
    """textnames renames every file through parameters.h's file-name macros:
    the host reads and writes the renamed files, as SCFT.c did."""
    build = importlib.import_module("stimuli-responsive-nanodroplets_gb300.build")
    gi = dict(np.load(GOLD / f"{inputs}.npz"))
    S = surface_from_json(srn, gi["surface"])
    d = srn.derive(S)
    (tmp_path / "parameters.h").write_text(S.to_parameters_h())
    exe = build.build_host(tmp_path)
    m3 = srn.configs.substrate_mask(S) if mask else None
    write_inputs(srn, d, S, gi["w0"], tmp_path, m3)
    r = subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    ref_dir = GOLD / f"text_{name}"
    for f in sorted(os.listdir(ref_dir)):
        assert (tmp_path / f).read_bytes() == (ref_dir / f).read_bytes(), f
    if name == "textnames":
        assert not (tmp_path / "counter.dat").exists() and not (tmp_path / "free_energy.dat").exists()


def test_c_host_volume_check(srn, tmp_path):
    build = importlib.import_module("stimuli-responsive-nanodroplets_gb300.build")
    s = srn.configs.bulk2d(nx=8, nz=8, iters=1)
    s.VOL_DBK = [0.9, 0.0, 0.0, 0.0]
    (tmp_path / "parameters.h").write_text(s.to_parameters_h())
    exe = build.build_host(tmp_path)
    r = subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 0
    want = (GOLD / "text_volfail" / "DENSITY_CHECK_FAIL.error").read_bytes()
    assert (tmp_path / "DENSITY_CHECK_FAIL.error").read_bytes() == want
