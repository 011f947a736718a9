"""The autotuner on the device: the first solve or assignment of a (kernel, shape, stencil) key times the
equivalent launch configurations and caches the fastest; later ones hit the cache; and every
configuration gives the same bits (the choices are forced through the cache file and compared with the
untuned run)."""
import numpy as np
import pytest

import common as cm
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

pytestmark = pytest.mark.gpu


@pytest.fixture
def fresh():
    api.tune_set_cache(None)
    api.tune_clear()
    yield
    api.tune_set_cache(None)
    api.tune_clear()


def _poisson(ctx, dims):
    D = len(dims)
    mesh = cm.mesh_uniform([n + 1 for n in dims])
    fd = cm.field_desc(D, capi.CENTER, [(capi.BC_NEUM, capi.BC_NEUM)] * D, ext=1)
    p = api.CartesianField(mesh, fd, ctx)
    f = api.CartesianField(mesh, fd, ctx)
    a = f.download()
    sl = f.index_slices([tuple(f.info.assignable[d]) for d in range(D)])
    v = np.random.default_rng(31).standard_normal(a[sl].shape)
    a[sl] = v - v.mean()
    f.upload(a)
    ops = [api.d2x, api.d2y, api.d2z][:D]
    getter = lambda e: f == sum((op(e) for op in ops[1:]), ops[0](e))

    def solve():
        p.assign(0.0)
        st = api.Solve(getter, p, api.StructSolverParams(tol=1e-10, maxIter=100, pinValue=True, precision="mixed"))
        assert st.converged
        return st.niter, st.relerr, p.download()
    return solve


def _same(a, b):
    assert a[0] == b[0] and a[1] == b[1] and np.array_equal(a[2], b[2])


def test_solver_choices_are_cached_and_change_no_bit(ctx, fresh, monkeypatch, tmp_path):
    cache = tmp_path / "tune.txt"
    # (3D: enough planes for z tiles, rows of a multiple of 4 cells for the staged smoother)
    solves = [_poisson(ctx, [128, 100, 96]), _poisson(ctx, [600, 450])]
    monkeypatch.setenv("OPFLOW_TUNE", "0")
    plain = [s() for s in solves]
    monkeypatch.delenv("OPFLOW_TUNE")
    api.tune_set_cache(cache)
    tuned = [s() for s in solves]
    for a, b in zip(plain, tuned):
        _same(a, b)
    lines = [ln.split() for ln in cache.read_text().splitlines()]
    keys = {ln[0]: int(ln[1]) for ln in lines}
    zkeys = [k for k in keys if k.startswith("mg_smooth_z/f32/")]
    tkeys = [k for k in keys if k.startswith("mg_tile/f32/")]
    assert zkeys and tkeys, keys
    assert all(keys[k] in (2, 4, 8, 16) for k in zkeys) and all(keys[k] in (0, 1) for k in tkeys)
    n_tuned, hits, entries = api.tune_stats()
    assert n_tuned == len(keys) == entries
    # the same shapes again: cache hits only
    for s in solves:
        s()
    assert api.tune_stats()[0] == n_tuned and api.tune_stats()[1] > hits
    # every other choice, forced through a cache file: the same bits
    for alt in range(3):  # plane batches 2 and 8, then the staged smoother (16)
        forced = tmp_path / ("forced%d.txt" % alt)
        forced.write_text("".join("%s %d 0\n" % (k, [2, 8, 16][alt] if k in zkeys else (1 - keys[k] if alt < 2 else keys[k])) for k in keys))
        api.tune_clear()
        api.tune_set_cache(forced)
        for a, s in zip(plain, solves):
            _same(a, s())
        assert api.tune_stats()[0] == 0  # nothing measured: every key came from the file


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_explicit_tiling_choice_changes_no_bit(ctx, fresh, monkeypatch, tmp_path, mode):
    monkeypatch.delenv("OPFLOW_AXIS_TILING", raising=False)
    # the tiling choice applies to the per-step fixed-point form: runs of several fixed-point steps on a
    # Dirichlet node grid otherwise keep the field in fixed point in a kernel of their own
    monkeypatch.setenv("OPFLOW_FX_RESIDENT", "0")
    dims, steps = (97, 43, 70), 4
    mesh = cm.mesh_uniform(list(dims))
    fd = cm.field_desc(3, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 3)
    hx = 1.0 / (dims[0] - 1)

    def run():
        u = api.CartesianField(mesh, fd, ctx)
        a = u.download()
        a[...] = 0.0
        sl = u.index_slices([tuple(u.info.assignable[d]) for d in range(3)])
        a[sl] = np.random.default_rng(78).random(a[sl].shape)
        u.upload(a)
        u.assign(cm.ftcs_expr(u, 0.1 * hx * hx, 3), steps=steps, mode=mode)
        return u.download()
    monkeypatch.setenv("OPFLOW_TUNE", "0")
    plain = run()
    monkeypatch.delenv("OPFLOW_TUNE")
    cache = tmp_path / "tune.txt"
    api.tune_set_cache(cache)
    assert np.array_equal(run(), plain)
    keys = {ln.split()[0]: int(ln.split()[1]) for ln in cache.read_text().splitlines()}
    akeys = [k for k in keys if k.startswith("axis3d/%s/" % ("fixed" if mode == "fast" else "exact"))]
    assert len(akeys) == 1 and keys[akeys[0]] in (0, 1), keys
    forced = tmp_path / "forced.txt"
    forced.write_text("%s %d 0\n" % (akeys[0], 1 - keys[akeys[0]]))
    api.tune_clear()
    api.tune_set_cache(forced)
    assert np.array_equal(run(), plain)
    assert api.tune_stats()[0] == 0


def test_batch_level_mixing_row_lengths_keeps_every_problem_smoothed(ctx, fresh, monkeypatch, tmp_path):
    """A batched level holding a problem with rows of 128 cells (staged tiles) and one with rows of 130
    (none): forcing the staged smoother there must still smooth both, so the results stay those of the
    untuned batch, bit for bit."""
    probs = [api.Problem([n, 96, 80], [1.0 / n, 1.0 / 96, 1.0 / 80], alpha=0.0, beta=1.0, loc=api.LocOnMesh.Center, bc=api.BCType.Neum)
             for n in (128, 130)]
    rng = np.random.default_rng(8)
    fs = []
    for p in probs:
        f = rng.standard_normal(int(np.prod(p.n)))
        fs.append(f - f.mean())

    def run():
        B = api.Batch(probs, api.StructSolverParams(tol=1e-10, maxIter=100, precision="mixed"), ctx)
        for i, f in enumerate(fs):
            B.set(i, f, np.zeros(f.size))
        st = B.solve()
        return [(s.niter, s.relerr) for s in st], [B.get(i) for i in range(len(probs))]
    monkeypatch.setenv("OPFLOW_TUNE", "0")
    plain = run()
    monkeypatch.delenv("OPFLOW_TUNE")
    cache = tmp_path / "tune.txt"
    api.tune_set_cache(cache)
    run()
    zkeys = [ln.split()[0] for ln in cache.read_text().splitlines() if ln.startswith("mg_smooth_z/f32/batch2/")]
    assert zkeys, cache.read_text()
    forced = tmp_path / "forced.txt"
    forced.write_text("".join("%s 16 0\n" % k for k in zkeys))
    api.tune_clear()
    api.tune_set_cache(forced)
    got = run()
    assert got[0] == plain[0]
    for a, b in zip(got[1], plain[1]):
        assert np.array_equal(a, b)
