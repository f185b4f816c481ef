"""Batching form: instances of one grid with different contour counts (NS), box
lengths (hence diffusion operators) and chi values in one context. Each
instance must give exactly the numbers of its own solo context — the
reductions run in a fixed order per instance and the operator tables are the
same ones a solo context builds."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mixed_surfaces(srn):
    base = [
        dict(ns=64, chi_ab=12.0, scale=1.0),
        dict(ns=80, chi_ab=20.0, scale=1.012),   # own operators (LX, LZ stretched, same grid)
        dict(ns=64, chi_ab=28.0, scale=1.0),     # shares instance 0's operators (same NS and box)
        dict(ns=101, chi_ab=24.0, scale=1.0),
        dict(ns=57, chi_ab=16.0, scale=0.99),
    ]
    out = []
    for p in base:
        s = srn.configs.film2d(nx=32, nz=16, ns=p["ns"], chi_ab=p["chi_ab"], iters=3)
        s.LX = 32 * 0.125 * p["scale"]
        s.LZ = 16 * 0.125 * p["scale"]
        out.append(s)
    return out


def _run(srn, surfaces, w, m, precision, kernel_path, n=3):
    with srn.Solver(surfaces, precision=precision, kernel_path=kernel_path) as sv:
        assert all(d.grid == sv.grid for d in sv.derived)
        for b in range(len(surfaces)):
            sv.set_fields(w, b)
            sv.set_masks(m, b)
            sv.set_iteration(1, b)
        outs = sv.iterate(n)
        phi = [sv.get_densities(b)[0] for b in range(len(surfaces))]
        wout = [sv.get_fields(b) for b in range(len(surfaces))]
    return outs, phi, wout


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("kernel_path", ["auto", "passes"])
def test_uneven_contour_counts_match_solo(srn, precision, kernel_path):
    surfaces = _mixed_surfaces(srn)
    ds = [srn.derive(s) for s in surfaces]
    assert len({int(d.ns_dbk[0]) for d in ds}) == 4            # four contour counts
    assert len({(d.alphax, d.alphaz) for d in ds}) == 4        # four operator sets for five instances
    w = srn.configs.droplet_fields(surfaces[0], seed=5, radius=1.2)
    m = srn.configs.substrate_mask(surfaces[0])
    outs, phi, wout = _run(srn, surfaces, w, m, precision, kernel_path)
    for b, s in enumerate(surfaces):
        o, p, wo = _run(srn, [s], w, m, precision, kernel_path)
        for k in range(len(outs)):
            assert o[k][0].free_energy == outs[k][b].free_energy, (b, k)
            assert o[k][0].rms == outs[k][b].rms, (b, k)
            np.testing.assert_array_equal(o[k][0].q, outs[k][b].q)
        np.testing.assert_array_equal(p[0], phi[b])
        np.testing.assert_array_equal(wo[0], wout[b])


def test_uneven_batch_fp64_matches_oracle(srn, oracle_mod):
    """The mixed batch in the plain form against the CPU restatement, per instance."""
    surfaces = _mixed_surfaces(srn)[:2]
    w = srn.configs.droplet_fields(surfaces[0], seed=6, radius=1.2)
    m = srn.configs.substrate_mask(surfaces[0])
    outs, phi, _ = _run(srn, surfaces, w, m, "fp64", "auto", n=2)
    for b, s in enumerate(surfaces):
        o = oracle_mod.Oracle(s)
        o.set_fields(w)
        o.set_masks(m)
        o.set_iter(1)
        rec = o.iterate(2)
        for k in range(2):
            f_ref = rec[k, 1]
            assert abs(outs[k][b].free_energy - f_ref) <= 1e-9 * max(1.0, abs(f_ref)), (b, k)
        ophi, _ = o.densities()
        scale = np.maximum(np.abs(ophi).max(axis=1, keepdims=True), 1e-300)
        assert np.all(np.abs(phi[b] - ophi) <= 1e-10 * scale + 1e-15), b
        o.close()


def test_mismatched_grid_is_rejected(srn):
    a = srn.configs.film2d(nx=32, nz=16, iters=2)
    b = srn.configs.film2d(nx=32, nz=24, iters=2)
    with pytest.raises(RuntimeError):
        srn.Solver([a, b])


def test_mismatched_species_is_rejected(srn):
    a = srn.configs.film2d(nx=32, nz=16, iters=2)
    b = srn.configs.film2d(nx=32, nz=16, iters=2)
    b.VOL_S = [0.05, 0.02, 0.0]
    with pytest.raises(RuntimeError):
        srn.Solver([a, b])


def _film(srn, nx, nz, ns, chi_ab, iters=400):
    s = srn.configs.film2d(nx=nx, nz=nz, ns=ns, chi_ab=chi_ab, iters=iters)
    return s


def test_stop_freezes_converged_instance(srn):
    """scft_set_stop: the instance that meets its tolerance is frozen (records
    repeat, fields stay), the other runs on exactly as it would alone."""
    s = srn.configs.bulk2d(nx=32, nz=32, iters=400)
    w = srn.configs.uniform_fields(s.grid(), seed=4, amp=0.1)
    with srn.Solver(s, precision="fp64") as solo:
        solo.set_fields(w)
        solo.set_iteration(1)
        pilot = [o[0] for o in solo.iterate(200)]
    # a tolerance first met at some iteration k <= 120 of the pilot run
    tol = min(r.rms for r in pilot[:121]) * (1.0 + 1e-9)
    k = next(i for i, r in enumerate(pilot) if r.rms < tol)
    with srn.Solver([s, s.copy()], precision="fp64") as sv:
        for b in range(2):
            sv.set_fields(w, b)
            sv.set_iteration(1, b)
        sv.set_stop(tol, instance=0)
        out = sv.iterate(200)
        w0 = sv.get_fields(0)
        rec0 = [o[0] for o in out]
        assert [r.converged for r in rec0].index(1) == k
        assert rec0[k].free_energy == pilot[k].free_energy
        assert all(r.converged and r.iter == rec0[k].iter and r.free_energy == rec0[k].free_energy
                   for r in rec0[k:])
        more = sv.iterate(5)
        np.testing.assert_array_equal(sv.get_fields(0), w0)
        assert more[-1][0].iter == rec0[k].iter
        last1 = more[-1][1]
    with srn.Solver(s, precision="fp64") as solo:
        solo.set_fields(w)
        solo.set_iteration(1)
        o = solo.iterate(205)
        assert o[-1][0].free_energy == last1.free_energy
        assert o[-1][0].iter == last1.iter
    # the frozen instance's state equals a solo run stopped at the same iteration
    with srn.Solver(s, precision="fp64") as solo:
        solo.set_fields(w)
        solo.set_iteration(1)
        solo.iterate(k + 1)
        np.testing.assert_array_equal(solo.get_fields(), w0)


def test_async_iterate_matches_sync(srn):
    s = _film(srn, 32, 16, 64, 18.0)
    w = srn.configs.droplet_fields(s, seed=2, radius=1.2)
    m = srn.configs.substrate_mask(s)
    res = []
    for mode in ("sync", "async"):
        with srn.Solver(s, precision="fp32", use_graph=True) as sv:
            sv.set_fields(w)
            sv.set_masks(m)
            sv.set_iteration(1)
            if mode == "sync":
                out = sv.iterate(40)
            else:
                sv.iterate_async(25)
                out = sv.iterate_wait()
                sv.iterate_async(15)
                out += sv.iterate_wait()
            res.append(([o[0].free_energy for o in out], sv.get_fields()))
    assert res[0][0] == res[1][0]
    np.testing.assert_array_equal(res[0][1], res[1][1])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_uneven_grids_match_solo(srn, precision):
    """A batch over two grids and three NS values: every instance equals its solo run."""
    batch_mod = __import__("importlib").import_module("stimuli-responsive-nanodroplets_gb300.batch")
    surfaces = [_film(srn, 32, 16, 64, 14.0), _film(srn, 24, 16, 80, 20.0), _film(srn, 32, 16, 90, 26.0),
                _film(srn, 24, 16, 64, 22.0)]
    inputs = [(srn.configs.droplet_fields(s, seed=20 + i, radius=1.0), srn.configs.substrate_mask(s))
              for i, s in enumerate(surfaces)]
    with batch_mod.Batch(surfaces, precision=precision, use_graph=True) as b:
        assert b.groups == 2
        for i, (w, m) in enumerate(inputs):
            b.set_fields(i, w)
            b.set_masks(i, m)
            b.set_iteration(i, 1)
        res = b.run(30, chunk=8)
        fields = [b.get_fields(i) for i in range(len(surfaces))]
    assert all(r.iterations == 30 and not r.converged for r in res)
    for i, s in enumerate(surfaces):
        with srn.Solver(s, precision=precision) as solo:
            solo.set_fields(inputs[i][0])
            solo.set_masks(inputs[i][1])
            solo.set_iteration(1)
            o = solo.iterate(30)
            assert o[-1][0].free_energy == res[i].free_energy, i
            np.testing.assert_array_equal(solo.get_fields(), fields[i])


def test_batch_run_to_tolerance(srn):
    batch_mod = __import__("importlib").import_module("stimuli-responsive-nanodroplets_gb300.batch")
    surfaces = [srn.configs.bulk2d(nx=32, nz=32, iters=2000), srn.configs.bulk2d(nx=48, nz=32, iters=2000)]
    fields = [srn.configs.uniform_fields(s.grid(), seed=i, amp=0.1) for i, s in enumerate(surfaces)]
    tols = []
    for s, w in zip(surfaces, fields):
        with srn.Solver(s, precision="fp32") as solo:
            solo.set_fields(w)
            solo.set_iteration(1)
            tols.append(min(o[0].rms for o in solo.iterate(150)) * 1.001)
    with batch_mod.Batch(surfaces, precision="fp32", use_graph=True) as b:
        for i, s in enumerate(surfaces):
            b.set_fields(i, fields[i])
            b.set_iteration(i, 1)
            b.set_stop(i, tols[i])
        res = b.run(1000, chunk=64)
        for i in range(2):
            _, tot = b.get_densities(i)
            assert res[i].converged and res[i].rms < tols[i] and res[i].iterations <= 150
            assert abs(np.sqrt(np.mean((tot - 1.0) ** 2)) - res[i].rms) <= 1e-12


def test_async_batched_transfers_match_sync(srn):
    """scft_*_all_async + scft_iterate_async / _wait give what the blocking calls give."""
    import ctypes as C
    import importlib
    L = importlib.import_module("stimuli-responsive-nanodroplets_gb300._lib")
    surfaces = [_film(srn, 32, 16, 50, 14.0 + 4 * b) for b in range(3)]
    w0 = np.stack([srn.configs.droplet_fields(s, seed=30 + b, radius=1.0) for b, s in enumerate(surfaces)])
    m = srn.configs.substrate_mask(surfaces[0])
    dp = C.POINTER(C.c_double)
    out = []
    for mode in ("sync", "async"):
        with srn.Solver(surfaces, precision="fp32", noise="device") as sv:
            for b in range(3):
                sv.set_masks(m, b)
                sv.set_iteration(1, b)
                sv.set_rng((b, 1, 2), b)
            w = np.ascontiguousarray(w0.copy())
            phi = np.zeros_like(w)
            lib = L.lib()
            for _ in range(4):
                if mode == "sync":
                    L.check(lib.scft_set_fields_all(sv._h, w.ctypes.data_as(dp)), "set")
                    sv.iterate(1)
                    L.check(lib.scft_get_fields_all(sv._h, w.ctypes.data_as(dp)), "get")
                    L.check(lib.scft_get_densities_all(sv._h, phi.ctypes.data_as(dp)), "getphi")
                else:
                    L.check(lib.scft_set_fields_all_async(sv._h, w.ctypes.data_as(dp)), "set")
                    sv.iterate_async(1)
                    L.check(lib.scft_get_fields_all_async(sv._h, w.ctypes.data_as(dp)), "get")
                    L.check(lib.scft_get_densities_all_async(sv._h, phi.ctypes.data_as(dp)), "getphi")
                    sv.iterate_wait()
            out.append((w.copy(), phi.copy()))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
