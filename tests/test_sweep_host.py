"""Hand-over logic of the precision form's finish (sweep.run_finished) on the
CPU: a fake batch stands in for the GPU one (same calls; an instance's RMS
falls geometrically to a floor that depends on the precision), so the FP32
phase, the hand-over on the floor, the finishing thread, the per-instance
iteration cap and the error path are checked without a device."""
import importlib
import math

import pytest

sweep = importlib.import_module("stimuli-responsive-nanodroplets_gb300.sweep")
batch_mod = importlib.import_module("stimuli-responsive-nanodroplets_gb300.batch")


class Spec:
    """Instance model: RMS r0 * g**k after k iterations, never below the
    precision's floor (floor32 in FP32, 0 in the finishing forms)."""

    def __init__(self, r0, g, floor32):
        self.r0, self.g, self.floor32 = r0, g, floor32


class FakeBatch:
    created = []

    def __init__(self, surfaces, precision="fp32", use_graph=True, noise="device", fail_after=None):
        self.specs = list(surfaces)
        self.n = len(self.specs)
        self.precision = precision
        self.rms = [s.r0 for s in self.specs]
        self.iter = [0] * self.n
        self.stop = [0.0] * self.n
        self.frozen = [False] * self.n
        self.fields_set = [False] * self.n
        self.runs = 0
        self.fail_after = fail_after
        self.closed = False
        self.armed_log = []
        FakeBatch.created.append(self)

    # --- the Batch calls run_finished uses
    def set_fields(self, i, w):
        self.fields_set[i] = True
        if isinstance(w, tuple) and w[0] == "rms":
            self.rms[i] = w[1]

    def set_masks(self, i, m):
        pass

    def set_iteration(self, i, it):
        self.iter[i] = it
        self.frozen[i] = False
        self.armed_log.append(i)

    def set_rng(self, i, seed):
        pass

    def set_stop(self, i, tol):
        self.stop[i] = tol

    def freeze(self, i):
        self.frozen[i] = True

    def get_fields(self, i):
        return ("rms", self.rms[i])

    def close(self):
        self.closed = True

    def run(self, max_iter, chunk=100):
        assert all(self.fields_set), "every instance needs fields before a run"
        self.runs += 1
        if self.fail_after is not None and self.runs > self.fail_after:
            raise RuntimeError("injected batch failure")
        out = []
        for i, s in enumerate(self.specs):
            if self.frozen[i]:
                out.append(batch_mod.BatchResult(0, self.iter[i], 1.0, self.rms[i], True, 0))
                continue
            floor = s.floor32 if self.precision == "fp32" else 0.0
            k = 0
            conv = False
            r = self.rms[i]
            while k < max_iter:
                r = max(r * s.g, floor)
                k += 1
                if r < self.stop[i]:
                    conv = True
                    break
            self.rms[i] = r
            self.iter[i] += k
            if conv:
                self.frozen[i] = True
            out.append(batch_mod.BatchResult(k, self.iter[i], 1.0 + r, r, conv, 0))
        return out


@pytest.fixture
def fake(monkeypatch):
    FakeBatch.created = []
    monkeypatch.setattr(sweep, "Batch", FakeBatch)
    return FakeBatch


def inputs(n):
    return [(None, None)] * n


def test_handover_converge_and_cap(fake):
    specs = [
        Spec(1e-2, 0.99, 5e-6),    # reaches the FP32 floor above 1e-6: handed over, converges
        Spec(1e-2, 0.99, 1e-8),    # no floor in reach: converges in FP32
        Spec(1e-2, 0.9999, 5e-6),  # too slow: hits the cap in FP32 (above the hand-over RMS)
        Spec(3e-5, 0.999, 6e-6),   # starts near the floor: handed over, capped in the finish
    ]
    res, wall, wall32 = sweep.run_finished(specs, inputs(4), rms_tol=1e-6, max_iter=3000, chunk=100,
                                           stall_round=200)
    fp32, fin = fake.created
    assert fp32.precision == "fp32" and fin.precision == "fp32x2"
    assert fp32.closed and fin.closed
    a, b, c, d = res
    # handed over on its floor, then converged in the finishing form within the cap
    assert a.converged and a.rms < 1e-6 and 0 < a.iterations_fp32 < a.iterations <= 3000
    # converged in FP32: no finishing iterations
    assert b.converged and b.iterations == b.iterations_fp32 and b.iterations <= 3000
    # capped in FP32, never handed over
    assert not c.converged and c.iterations == c.iterations_fp32 >= 3000
    assert 2 not in fin.armed_log
    # handed over, capped in the finishing form: counted as not converged
    assert not d.converged and d.iterations >= 3000 and d.iterations_fp32 < d.iterations
    assert sorted(fin.armed_log) == [0, 3]
    assert 0 <= wall32 <= wall


def test_finish_precision_choice(fake):
    specs = [Spec(1e-2, 0.99, 5e-6)]
    res, _, _ = sweep.run_finished(specs, inputs(1), rms_tol=1e-6, max_iter=5000, finish="fp64")
    assert fake.created[1].precision == "fp64"
    assert res[0].converged


def test_fp32_failure_stops_the_finisher(fake, monkeypatch):
    orig = FakeBatch.__init__

    def init(self, surfaces, precision="fp32", use_graph=True, noise="device"):
        orig(self, surfaces, precision, use_graph, noise, fail_after=3 if precision == "fp32" else None)

    monkeypatch.setattr(FakeBatch, "__init__", init)
    specs = [Spec(1e-2, 0.98, 5e-6), Spec(1e-2, 0.9999, 5e-6)]
    with pytest.raises(RuntimeError, match="injected"):
        sweep.run_finished(specs, inputs(2), rms_tol=1e-6, max_iter=100000, chunk=100, stall_round=100)
    fp32, fin = fake.created
    assert fp32.closed and fin.closed


def test_finisher_failure_is_reported(fake, monkeypatch):
    orig = FakeBatch.__init__

    def init(self, surfaces, precision="fp32", use_graph=True, noise="device"):
        orig(self, surfaces, precision, use_graph, noise, fail_after=0 if precision != "fp32" else None)

    monkeypatch.setattr(FakeBatch, "__init__", init)
    specs = [Spec(1e-2, 0.99, 5e-6), Spec(1e-2, 0.9999, 5e-6)]
    with pytest.raises(RuntimeError, match="injected"):
        sweep.run_finished(specs, inputs(2), rms_tol=1e-6, max_iter=20000, chunk=100, stall_round=200)
    assert all(b.closed for b in fake.created)


def test_model_floor_is_reached():
    # the fake's FP32 floor sits between the tolerance and the hand-over RMS,
    # as the measured FP32 floor (3e-6 - 9e-6) does
    assert 1e-6 < 5e-6 < sweep.SWITCH_RMS
    assert math.log(5e-6 / 1e-2) / math.log(0.99) < 3000
