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
