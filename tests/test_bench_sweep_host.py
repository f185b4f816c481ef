"""The sweep record of bench.py on the CPU: fake batches stand in for the GPU
ones, so every form, the diagonal subset, the full point set, the solves/hour
ratios and the free-energy agreement between forms are checked without a
device."""
import importlib
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

sweep = importlib.import_module("stimuli-responsive-nanodroplets_gb300.sweep")
batch_mod = importlib.import_module("stimuli-responsive-nanodroplets_gb300.batch")
srn = importlib.import_module("stimuli-responsive-nanodroplets_gb300")


class FakeSweepBatch:
    """Instance k of a form converges when (k + offset) is even; F = 10 + k (+ a
    form-dependent error), RMS 1e-7 if converged, 1e-5 otherwise."""

    F_ERR = {"fp32": 2e-7, "fp64": 0.0, "fp32x2": 1e-14}

    def __init__(self, surfaces, precision):
        self.surfaces, self.precision = surfaces, precision
        self.groups = 2

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def run(self, max_iter, chunk=200):
        out = []
        for k, s in enumerate(self.surfaces):
            conv = (s.fake_id % 2 == 0) or self.precision != "fp32"
            F = (10.0 + s.fake_id) * (1.0 + self.F_ERR[self.precision])
            out.append(batch_mod.BatchResult(100 + k, 101 + k, F, 1e-7 if conv else 1e-5, conv, 0))
        return out


@pytest.fixture
def fakes(monkeypatch):
    real_surfaces = srn.configs.sweep_surfaces

    def surfaces(n, **kw):
        ss = real_surfaces(n, **kw)
        for i, s in enumerate(ss):
            s.fake_id = i
        return ss

    monkeypatch.setattr(srn.configs, "sweep_surfaces", surfaces)
    monkeypatch.setattr(sweep, "sweep_inputs", lambda ss: [(None, None)] * len(ss))
    monkeypatch.setattr(sweep, "make_batch", lambda ss, si, prec, tol, use_graph=True: FakeSweepBatch(ss, prec))

    def run_finished(ss, si, rms_tol, max_iter, finish="fp32x2", **kw):
        res = [sweep.FinishedResult(300, 200, 1e-7, (10.0 + s.fake_id) * (1.0 + 3e-13), True, 0) for s in ss]
        return res, 2.0, 1.0

    monkeypatch.setattr(sweep, "run_finished", run_finished)


def _bench():
    import bench
    return bench


def test_sweep_record_below_the_floor(fakes):
    bench = _bench()
    out = bench.measure_sweep(srn, 4, 1e-6, 1000, 4, 0, lambda: None, keep_points=True)
    sub = out["subset"]
    assert out["fp32"]["instances"] == 16 and "final_free_energy" in out["fp32"]
    assert len(sub["points"]) == 4
    for key in ("fp32", "fp64_plain", "fp32x2", "fp32_fp32x2_finish", "fp32_fp64_finish"):
        assert key in sub, key
    # FP32 converges the even points only; the FP64 form all four
    assert sub["fp64_plain"]["converged"] == 4
    assert sub["fp32_vs_fp64_converged_in_both"] == sub["fp32"]["converged"]
    assert sub["fp32_vs_fp64_max_rel_free_energy_diff"] == pytest.approx(2e-7, rel=1e-6)
    fin = sub["fp32_fp32x2_finish"]
    assert fin["converged"] == 4 and fin["converged_in_both"] == 4
    assert fin["max_rel_free_energy_diff_vs_fp64"] == pytest.approx(3e-13, rel=1e-3)
    assert sub["solves_per_hour_ratio_fp32x2_finish_over_fp64"] == pytest.approx(
        fin["solves_per_hour"] / sub["fp64_plain"]["solves_per_hour"])


def test_sweep_record_full_set_and_form_choice(fakes):
    bench = _bench()
    out = bench.measure_sweep(srn, 2, 1e-6, 1000, 4, 0, lambda: None, keep_points=False,
                              forms=("finish_fp32x2",))
    sub = out["subset"]
    assert sub["points"] == "all" and sub["fp32"] is out["fp32"]
    assert "fp64_plain" not in sub and "fp32x2" not in sub and "fp32_fp64_finish" not in sub
    fin = sub["fp32_fp32x2_finish"]
    assert fin["converged"] == 4 and "converged_in_both" not in fin
    assert "final_rms" not in out["fp32"] and "final_free_energy" not in out["fp32"]


def test_sweep_record_above_the_floor(fakes):
    bench = _bench()
    out = bench.measure_sweep(srn, 4, 1e-4, 1000, 4, 0, lambda: None)
    sub = out["subset"]
    assert "fp32x2" not in sub and "fp32_fp32x2_finish" not in sub
    assert sub["solves_per_hour_ratio_fp32_over_fp64"] > 0
    assert "final_rms" not in sub["fp32"] and "final_free_energy" not in sub["fp64_plain"]
