"""End-to-end workflows on the GPU at small sizes: the droplet sweep over
uneven grids run to a tolerance, and the phase-diagram passes on top of the
serving loop (FP32 winners confirmed by the plain FP64 form)."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sweep = importlib.import_module("stimuli-responsive-nanodroplets_gb300.sweep")
serve = importlib.import_module("stimuli-responsive-nanodroplets_gb300.serve")
phase = importlib.import_module("stimuli-responsive-nanodroplets_gb300.phase")


def test_small_sweep_runs_to_tolerance(srn):
    run = sweep.run_sweep(n=2, precision="fp32", rms_tol=5e-3, max_iter=600, chunk=50, seed=1,
                          sizes=((32, 16), (48, 16)), ns_range=(40, 60))
    st = sweep.summary(run)
    assert st["instances"] == 4 and st["groups"] == 2
    for r in run.results:
        assert r.status == 0 and np.isfinite(r.free_energy)
        if r.converged:
            assert r.rms < 5e-3 and r.iterations <= 600
    assert st["converged"] >= 1


@pytest.mark.parametrize("finish", ["fp32x2", "fp64"])
def test_fp32_with_finish_reaches_the_fp64_fixed_point(srn, finish):
    """Below the FP32 form's RMS floor the precision form hands each instance
    over to a finishing form (double-float or plain FP64 propagators): it
    converges to the tolerance, to the free energy the plain FP64 form reaches
    on its own (1e-6 relative), having run its first iterations in FP32,
    within its own iteration cap."""
    cfg = srn.configs
    surfaces = cfg.sweep_surfaces(2, seed=1, sizes=((32, 16), (48, 16)), ns_range=(40, 60))
    inputs = sweep.sweep_inputs(surfaces)
    # hand-over forced above the tolerance (floor_rms), so both phases run
    res, wall, wall32 = sweep.run_finished(surfaces, inputs, rms_tol=1e-5, max_iter=8000, switch_rms=1e-4,
                                           floor_rms=5e-5, finish=finish)
    with sweep.make_batch(surfaces, inputs, "fp64", 1e-5) as b:
        ref = b.run(8000, chunk=200)
    assert 0 < wall32 < wall
    for r, f in zip(res, ref):
        assert r.status == 0 and f.converged
        assert r.converged and r.rms < 1e-5 and 0 < r.iterations_fp32 < r.iterations
        assert abs(r.free_energy - f.free_energy) <= 1e-6 * abs(f.free_energy)


def _film(cfg, p, chi_ab, chi_ac, prec_ns=40):
    return cfg.film_point(chi_ab, chi_ac, cfg.PLANES[p], nx=32, nz=16, ns=prec_ns)


def test_phase_diagram_passes_and_fp64_winners(srn, tmp_path):
    cfg = srn.configs
    n = 2
    ab, ac = cfg.chi_axes(n, ab=(12.0, 20.0), ac=(25.0, 40.0))
    kinds = ("lamellar", "cylinder", "disordered")

    def surface_fn(p):
        return _film(cfg, p[0], float(ab[p[1]]), float(ac[p[2]]))

    def seed_fn(p):
        s = surface_fn(p)
        return cfg.seed_fields(s, kinds[(p[0] + p[1] + p[2]) % 3], seed=7 + p[1] * n + p[2]), cfg.substrate_mask(s)

    tmpl = surface_fn((0, 0, 0))
    pools = {("film", "fp32"): serve.Pool("film", tmpl, 8, "fp32")}
    server = serve.Server(pools, rms_tol=5e-3, max_iter=300, chunk=50)
    pd = phase.PhaseDiagram(server, "film", "fp32", n, surface_fn, seed_fn, planes=3, outdir=tmp_path)
    passes = pd.run(max_passes=4)
    server.close()
    assert passes >= 2
    F = pd.free_energies()
    assert np.isfinite(F).all()
    assert len(list(tmp_path.glob("P*_*_*.json"))) == 3 * n * n
    # every point ends at the lowest free energy among the trials it ran
    for p, st in pd.state.items():
        tried = [f for (q, src, f, conv) in pd.trials if q == p and np.isfinite(f)]
        assert st.free_energy == min(tried)
    # the FP64 plain form picks the same winner at a point with a replacement
    replaced = [p for p, st in pd.state.items() if st.history]
    if replaced:
        p = replaced[0]
        # relax the point's own seed and its winning converged field in both forms
        winner_field = pd.state[p].fields
        s = surface_fn(p)
        m = cfg.substrate_mask(s)
        res = {}
        for prec in ("fp32", "fp64"):
            with srn.Solver([s, s.copy()], precision=prec) as sv:
                for b, w in enumerate((seed_fn(p)[0], winner_field)):
                    sv.set_fields(w, b)
                    sv.set_masks(m, b)
                    sv.set_iteration(1, b)
                out = sv.iterate(300)
                res[prec] = [out[-1][b].free_energy for b in range(2)]
        assert int(np.argmin(res["fp32"])) == int(np.argmin(res["fp64"]))
