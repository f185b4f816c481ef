"""Serving loop on the GPU: continuous batching with slot reuse gives every
request exactly the result it gets alone (same iterations, free energy and
fields, bit for bit), for both shape classes and both precisions."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

serve = importlib.import_module("stimuli-responsive-nanodroplets_gb300.serve")


def _requests(srn, n_film=6, n_bulk=3):
    cfg = srn.configs
    reqs = []
    kinds = ("lamellar", "cylinder", "disordered")
    for r in range(n_film):
        plane = cfg.PLANES[r % 3]
        s = cfg.film_point(12.0 + 3.0 * r, 25.0 + 5.0 * r, plane, nx=32, nz=16, ns=60)
        reqs.append(serve.Request(rid=r, cls="film", surface=s, w14=cfg.seed_fields(s, kinds[r % 3], seed=r),
                                  mask3=cfg.substrate_mask(s), precision="fp32" if r % 2 == 0 else "fp64",
                                  arrival=0.0, key=("film", r), seed=(r, 1, 2)))
    for r in range(n_bulk):
        s = cfg.bulk3d_point(15.0 + 4.0 * r, 30.0, cfg.PLANES[r % 3], n=16, ns=40)
        reqs.append(serve.Request(rid=100 + r, cls="bulk", surface=s, w14=cfg.seed_fields(s, kinds[r], seed=r),
                                  precision="fp32", key=("bulk", r)))
    return reqs


def _pools(srn, film_slots, bulk_slots):
    cfg = srn.configs
    ft = cfg.film_point(20.0, 40.0, cfg.PLANES[0], nx=32, nz=16, ns=60)
    bt = cfg.bulk3d_point(20.0, 40.0, cfg.PLANES[0], n=16, ns=40)
    return {("film", "fp32"): serve.Pool("film", ft, film_slots, "fp32"),
            ("film", "fp64"): serve.Pool("film", ft, film_slots, "fp64"),
            ("bulk", "fp32"): serve.Pool("bulk", bt, bulk_slots, "fp32")}


def test_results_same_alone_and_in_the_mix(srn):
    reqs = _requests(srn)
    server = serve.Server(_pools(srn, 2, 2), rms_tol=2e-3, max_iter=120, chunk=20, keep_fields=True)
    mixed = {c.rid: c for c in server.run(reqs, realtime=False)}
    server.close()
    assert len(mixed) == len(reqs)
    for r in reqs:
        alone_server = serve.Server(_pools(srn, 1, 1), rms_tol=2e-3, max_iter=120, chunk=20, keep_fields=True)
        alone = alone_server.run([r], realtime=False)[0]
        alone_server.close()
        m = mixed[r.rid]
        assert (alone.iterations, alone.converged) == (m.iterations, m.converged), r.rid
        assert alone.free_energy == m.free_energy, r.rid
        np.testing.assert_array_equal(alone.fields, m.fields)


def test_realtime_poisson_stream_reports_latency(srn):
    reqs = _requests(srn, n_film=4, n_bulk=2)
    rng = np.random.default_rng(0)
    t = np.cumsum(rng.exponential(0.05, len(reqs)))
    for r, a in zip(reqs, t):
        r.arrival = float(a)
    server = serve.Server(_pools(srn, 2, 1), rms_tol=2e-3, max_iter=100, chunk=20)
    import time
    t0 = time.perf_counter()
    done = server.run(reqs)
    wall = time.perf_counter() - t0
    server.close()
    st = serve.latency_stats(done, wall)
    assert st["requests"] == len(reqs)
    assert all(c.finished >= c.admitted >= c.arrival - 1e-9 for c in done)
    assert 0.0 < st["p50_s"] <= st["p99_s"] <= wall


def _film(srn, r, bad=None):
    """A thin-film request; bad = "nan" puts NaN into its A field, "overflow"
    makes exp(-w ds/2) overflow the FP32 propagator within a few steps."""
    cfg = srn.configs
    s = cfg.film_point(12.0 + 3.0 * r, 25.0 + 5.0 * r, cfg.PLANES[r % 3], nx=32, nz=16, ns=60)
    w = cfg.seed_fields(s, ("lamellar", "cylinder", "disordered")[r % 3], seed=r)
    if bad == "nan":
        w = w.copy()
        w[0, 5] = np.nan
    elif bad == "overflow":
        w = w.copy()
        w[0, :] = -4000.0
    return serve.Request(rid=r, cls="film", surface=s, w14=w, mask3=cfg.substrate_mask(s), precision="fp32",
                         key=("film", r), seed=(r, 1, 2))


def _film_pool(srn, slots):
    cfg = srn.configs
    ft = cfg.film_point(20.0, 40.0, cfg.PLANES[0], nx=32, nz=16, ns=60)
    return {("film", "fp32"): serve.Pool("film", ft, slots, "fp32")}


def test_host_injected_nonfinite_requests(srn):
    """Fault injection from the host: requests whose fields are NaN or overflow
    the FP32 propagator end with SCFT_ERR_NONFINITE; their slots take the next
    requests, and every other request comes out bit for bit as it does alone."""
    L = importlib.import_module("stimuli-responsive-nanodroplets_gb300._lib")
    reqs = [_film(srn, 0, "nan"), _film(srn, 1), _film(srn, 2, "overflow"), _film(srn, 3), _film(srn, 4),
            _film(srn, 5, "nan"), _film(srn, 6)]
    server = serve.Server(_film_pool(srn, 2), rms_tol=2e-3, max_iter=120, chunk=20, keep_fields=True)
    mixed = {c.rid: c for c in server.run(reqs, realtime=False)}
    server.close()
    assert sorted(mixed) == [r.rid for r in reqs]
    for r in reqs:
        m = mixed[r.rid]
        if r.rid in (0, 2, 5):
            assert m.status == L.ERR_NONFINITE and not m.converged, r.rid
            assert m.iterations <= 20, r.rid  # ended at the first chunk boundary
            continue
        assert m.status == 0, r.rid
        alone_server = serve.Server(_film_pool(srn, 1), rms_tol=2e-3, max_iter=120, chunk=20, keep_fields=True)
        alone = alone_server.run([r], realtime=False)[0]
        alone_server.close()
        assert (alone.iterations, alone.converged, alone.status) == (m.iterations, m.converged, m.status), r.rid
        assert alone.free_energy == m.free_energy, r.rid
        np.testing.assert_array_equal(alone.fields, m.fields)


def test_memory_budget_admission(srn):
    """Admission by memory: a budget below one slot is refused, and a budget
    above the device's memory is capped by what is free."""
    cfg = srn.configs
    ft = cfg.film_point(20.0, 40.0, cfg.PLANES[0], nx=32, nz=16, ns=60)
    with pytest.raises(serve.BudgetError):
        serve.slots_for_budget(ft, "fp32", 1024)
    free, total = importlib.import_module("stimuli-responsive-nanodroplets_gb300.solver").device_memory(0)
    assert 0 < free <= total
    n = serve.slots_for_budget(ft, "fp32", 100 * total, max_slots=10 ** 9)
    with srn.Solver([ft, ft], precision="fp32") as two, srn.Solver([ft], precision="fp32") as one:
        per_slot = two.device_bytes - one.device_bytes
    assert n * per_slot <= free

