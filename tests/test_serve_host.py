"""Scheduler logic of the serving loop on the CPU: a fake context stands in
for the GPU one (same calls, instance i converges after a fixed number of
iterations), so admission, slot reuse, freezing and completion order are
checked without a device."""
import importlib

import numpy as np
import pytest

serve = importlib.import_module("stimuli-responsive-nanodroplets_gb300.serve")
srn = importlib.import_module("stimuli-responsive-nanodroplets_gb300")


class FakeRec:
    def __init__(self, it, conv, F, status=0):
        self.iter, self.converged, self.free_energy, self.rms, self.status = it, conv, F, 0.0 if conv else 1.0, status


class FakeSolver:
    """Slot b of request r converges after need[r] iterations; a negative
    need[r] fails (status SCFT_ERR_NONFINITE) after -need[r] iterations."""

    def __init__(self, slots, need):
        self.B, self.need, self.M = slots, need, 8
        self.it = [1] * slots
        self.frozen = [True] * slots
        self.req = [None] * slots
        self.pending = 0
        self.log = []

    device_bytes = 1

    def set_surface(self, b, s):
        self.req[b] = s.rid

    def set_fields(self, w, b):
        assert self.frozen[b]

    def set_masks(self, m, b):
        pass

    def set_rng(self, seed, b):
        pass

    def set_stop(self, tol, b):
        pass

    def set_iteration(self, it, b):
        self.it[b] = it
        self.frozen[b] = self.req[b] is None

    def freeze(self, b):
        self.frozen[b] = True

    def iterate_async(self, n):
        assert not self.pending
        self.pending = n

    def iterate_ready(self):
        return True

    def iterate_wait(self, allow_nonfinite=False):
        n, self.pending = self.pending, 0
        recs, failed = [], False
        for _ in range(n):
            row = []
            for b in range(self.B):
                need = self.need[self.req[b]] if self.req[b] is not None else 0
                if not self.frozen[b]:
                    self.it[b] += 1
                    if self.it[b] - 1 >= abs(need):
                        self.frozen[b] = True
                        self.log.append((self.req[b], self.it[b] - 1))
                bad = self.frozen[b] and need < 0 and self.it[b] - 1 >= -need
                failed |= bad
                row.append(FakeRec(self.it[b], self.frozen[b] and self.req[b] is not None and not bad,
                                   float(self.req[b] or 0), -4 if bad else 0))
            recs.append(row)
        if failed and not allow_nonfinite:
            raise RuntimeError("SCFT_ERR_NONFINITE")
        return recs

    def get_fields(self, b):
        return np.zeros((14, self.M))

    def close(self):
        pass


class Tagged:
    def __init__(self, rid):
        self.rid = rid


def make_requests(need):
    return [serve.Request(rid=i, cls="c", surface=Tagged(i), w14=np.zeros((14, 8)), precision="fp32", key=(i,))
            for i in range(len(need))]


def test_slots_are_reused_and_every_request_completes():
    need = [30, 75, 10, 50, 20, 90, 15, 40]
    fake = FakeSolver(3, need)
    pool = serve.Pool("c", None, 3, "fp32", solver=fake)
    server = serve.Server({("c", "fp32"): pool}, rms_tol=1e-6, max_iter=1000, chunk=10)
    done = server.run(make_requests(need), realtime=False)
    assert sorted(c.rid for c in done) == list(range(len(need)))
    for c in done:
        # a request finishes at the first chunk boundary after it converged
        assert c.converged and c.iterations == need[c.rid]
    assert not pool.busy and sorted(pool.free) == [0, 1, 2]
    # with 3 slots, request 3 could start only after one of 0..2 finished
    order = [c.rid for c in sorted(done, key=lambda c: c.finished)]
    assert order.index(2) < order.index(5)


def test_max_iter_ends_unconverged_requests():
    need = [500, 20]
    fake = FakeSolver(2, need)
    pool = serve.Pool("c", None, 2, "fp32", solver=fake)
    server = serve.Server({("c", "fp32"): pool}, max_iter=100, chunk=25)
    done = {c.rid: c for c in server.run(make_requests(need), realtime=False)}
    assert not done[0].converged and done[0].iterations == 100
    assert done[1].converged and done[1].iterations == 20


def test_unknown_class_is_rejected():
    pool = serve.Pool("c", None, 1, "fp32", solver=FakeSolver(1, [1]))
    server = serve.Server({("c", "fp32"): pool})
    r = make_requests([1])[0]
    r.cls = "other"
    with pytest.raises(KeyError):
        server.run([r])


def test_latency_stats():
    cs = [serve.Completion(i, (), "c", "fp32", 0.0, 0.0, float(i + 1), 10, 0.0, 0.0, True, 0) for i in range(100)]
    st = serve.latency_stats(cs, wall_s=100.0)
    assert st["p50_s"] == pytest.approx(50.5) and st["p99_s"] == pytest.approx(99.01)
    assert st["solves_per_hour"] == pytest.approx(3600.0)


def test_plane_surfaces_share_shape_within_a_class():
    cfg = srn.configs
    a = cfg.film_point(10.0, 20.0, cfg.PLANES[0], nx=32, nz=16)
    b = cfg.film_point(30.0, 60.0, cfg.PLANES[2], nx=32, nz=16)
    da, db = srn.derive(a), srn.derive(b)
    assert da.grid == db.grid and da.alphax == db.alphax and list(da.active) == list(db.active)
    c = cfg.bulk3d_point(10.0, 20.0, cfg.PLANES[1], n=16)
    assert srn.derive(c).grid == (16, 16, 16)
    for kind in ("lamellar", "cylinder", "disordered"):
        w = cfg.seed_fields(a, kind, seed=1)
        assert w.shape == (14, 32 * 16) and np.isfinite(w).all()


def test_failed_request_ends_alone_and_frees_its_slot():
    """A request whose instance turns non-finite completes with that status at
    the next chunk boundary; its slot takes the next request, and every other
    request completes as it would without it."""
    need = [40, -15, 30, -5, 25, 35]
    fake = FakeSolver(2, need)
    pool = serve.Pool("c", None, 2, "fp32", solver=fake)
    server = serve.Server({("c", "fp32"): pool}, rms_tol=1e-6, max_iter=1000, chunk=10)
    done = {c.rid: c for c in server.run(make_requests(need), realtime=False)}
    assert sorted(done) == list(range(len(need)))
    for rid, n in enumerate(need):
        c = done[rid]
        if n < 0:
            assert c.status == -4 and not c.converged and c.iterations == -n
        else:
            assert c.status == 0 and c.converged and c.iterations == n
    assert not pool.busy and sorted(pool.free) == [0, 1]
    # the two slots served all six requests: failed slots were reused
    assert len({r for r, _ in fake.log}) == len(need)

