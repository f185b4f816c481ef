"""Phase-diagram driver logic on the CPU with a fake server: neighbour sets,
trial bookkeeping, lowest-F replacement, history and per-point JSON records."""
import importlib
import json

import numpy as np

phase = importlib.import_module("stimuli-responsive-nanodroplets_gb300.phase")
serve = importlib.import_module("stimuli-responsive-nanodroplets_gb300.serve")


def test_neighbours():
    assert sorted(phase.neighbours((0, 0, 0), 3)) == [(0, 0, 1), (0, 1, 0), (1, 0, 0), (2, 0, 0)]
    assert len(phase.neighbours((1, 1, 1), 3)) == 6
    assert sorted(phase.neighbours((2, 1, 1), 3, planes=3))[0] == (0, 1, 1)
    assert len(phase.neighbours((0, 1, 1), 3, planes=1)) == 4


class FakeServer:
    """A structure is identified by the integer tag in w14[0, 0]; the free energy of
    tag t at point p is energy(p, t). A solve keeps the tag (the converged field
    is the seed's structure)."""

    def __init__(self, energy):
        self.energy, self.keep_fields, self.calls = energy, False, 0

    def run(self, reqs, realtime=False):
        self.calls += 1
        out = []
        for r in reqs:
            tag = int(r.w14[0, 0])
            p = r.key[0]
            out.append(serve.Completion(r.rid, r.key, r.cls, r.precision, 0.0, 0.0, 0.0, 10,
                                        self.energy(p, tag), 0.0, True, 0, r.w14.copy()))
        return out


def test_lowest_free_energy_spreads_and_loop_stops(tmp_path):
    n = 3
    # structure tag = 1 + plane*9 + i*3 + j (each point starts with its own); tag 5 is
    # the best everywhere in plane 0, plane-0 structures beat other planes' structures
    def energy(p, tag):
        return 0.0 if tag == 5 else 1.0 + 0.01 * tag

    def seed(p):
        w = np.zeros((14, 4))
        w[0, 0] = 1 + p[0] * 9 + p[1] * 3 + p[2]
        return w, None

    srv = FakeServer(energy)
    pd = phase.PhaseDiagram(srv, "c", "fp32", n, surface_fn=lambda p: None, seed_fn=seed, outdir=tmp_path)
    passes = pd.run(max_passes=20)
    F = pd.free_energies()
    # tag 5 starts at (0,1,1) and reaches every point through neighbour trials
    assert np.all(F == 0.0)
    assert passes < 20
    rec = json.loads((tmp_path / "P2_0_0.json").read_text())
    assert rec["free_energy"] == 0.0 and rec["history"] and rec["history"][0]["source"] == "initial"
    assert {m.split("@")[0] for m in rec["tried"]} <= set(rec["neighbours"])
    # every (point, neighbour state) pair is tried at most once
    assert all(len(st.tried) == len(set(st.tried)) for st in pd.state.values())


def test_no_replacement_when_initial_is_best():
    def energy(p, tag):
        own = 1 + p[0] * 4 + p[1] * 2 + p[2]
        return 0.0 if tag == own else 1.0

    def seed(p):
        w = np.zeros((14, 4))
        w[0, 0] = 1 + p[0] * 4 + p[1] * 2 + p[2]
        return w, None

    pd = phase.PhaseDiagram(FakeServer(energy), "c", "fp32", 2, surface_fn=lambda p: None, seed_fn=seed)
    assert pd.run() == 2  # first pass + one pass without replacements
    assert all(st.source == "initial" and not st.history for st in pd.state.values())
