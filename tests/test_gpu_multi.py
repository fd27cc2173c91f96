"""GPU: several meshes of uneven size (and uneven signal counts) in one
persistent launch (bt_solve_multi) against the FP64 path mesh by mesh.
Tolerance: 1e-6 relative signal error, the mixed path's accuracy."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIX_RTOL = 1e-6


def contexts(pkg, meshes):
    pg = pkg.sequences.pgse(10600, 43100)
    og = pkg.sequences.cos_ogse(10600, 43100)
    (fn0, fo0), (fn1, fo1) = (pkg.sequences.profile_samples(p, 200.0) for p in (pg, og))
    out = []
    for m in meshes:
        ctx = pkg.Context(0)
        ctx.mesh_upload(m["xyz"], m["tets"], m["region"], 2)
        ctx.set_coefficients(m["D"], None, m["kappa"])
        ctx.assemble()
        ctx.set_schedule(np.array([fn0, fn1]), np.array([fo0, fo1]), 200.0)
        out.append(ctx)
    return out, [pg.int4gb(), og.int4gb()]


def test_uneven_meshes_one_launch_match_fp64(pkg, lib):
    meshes = pkg.meshgen.uneven_meshes(count=4, seed=3, nmin=6, nmax=14, cube=1.5)
    ctxs, int4 = contexts(pkg, meshes)
    counts = [3, 8, 1, 5]
    rng = np.random.default_rng(7)
    q, g, sq = [], [], []
    for c in counts:
        dirs = rng.normal(size=(c, 3))
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        seqs = rng.integers(0, 2, size=c)
        b = rng.uniform(500, 4000, size=c)
        q.append([pkg.sequences.b_to_q(bb, int4[s]) for bb, s in zip(b, seqs)])
        g.append(dirs)
        sq.append(seqs)
    out = pkg.solve_multi(ctxs, q, g, sq, rtol=1e-9)
    assert out["stats"]["total_iterations"] > 0
    for m, ctx in enumerate(ctxs):
        ref = ctx.solve(q[m], g[m], sq[m], precision=pkg.PRECISION_FP64, rtol=1e-12)
        rel = np.abs(out["signal"][m] - ref["signal"]) / np.abs(ref["signal"])
        assert rel.max() <= MIX_RTOL, (m, rel.max())
        assert abs(out["S0"][m] - ref["S0"]) <= 1e-12 * ref["S0"]
    # the same batch again: bitwise reproducible
    again = pkg.solve_multi(ctxs, q, g, sq, rtol=1e-9)
    for a, b in zip(out["signal"], again["signal"]):
        assert np.array_equal(a, b)
    for c in ctxs:
        c.close()


def test_multi_rejects_bad_calls(pkg, lib):
    meshes = pkg.meshgen.uneven_meshes(count=2, seed=1, nmin=5, nmax=6, cube=1.5)
    ctxs, int4 = contexts(pkg, meshes)
    q = [[pkg.sequences.b_to_q(1000.0, int4[0])]] * 2
    g = [[[1.0, 0.0, 0.0]]] * 2
    with pytest.raises(pkg.BtError) as e:
        pkg.solve_multi([ctxs[0], ctxs[0]], q, g)          # one context twice
    assert e.value.code == 1
    fresh = pkg.Context(0)
    m = meshes[1]
    fresh.mesh_upload(m["xyz"], m["tets"], m["region"], 2)
    with pytest.raises(pkg.BtError) as e:
        pkg.solve_multi([ctxs[0], fresh], q, g)             # not assembled
    assert e.value.code == 7
    with pytest.raises(pkg.BtError):
        pkg.solve_multi(ctxs, q, g, [[0], [5]])            # no such sequence row
    for c in ctxs + [fresh]:
        c.close()


def test_large_and_small_meshes_together(pkg, lib):
    """One mesh large enough to fill the GPU runs on its own, the small ones share
    a launch; every signal still matches the FP64 path."""
    big = pkg.meshgen.workload("cfg2", n=30)
    small = pkg.meshgen.uneven_meshes(count=2, seed=5, nmin=6, nmax=8, cube=1.5)
    meshes = [dict(xyz=big["xyz"], tets=big["tets"], region=big["region"], D=big["D"], kappa=big["kappa"])] + small
    ctxs, int4 = contexts(pkg, meshes)
    q = [[pkg.sequences.b_to_q(b, int4[0]) for b in (1000.0, 2000.0, 3000.0, 4000.0)]] * 3
    g = [pkg.meshgen.fibonacci_directions(4)] * 3
    out = pkg.solve_multi(ctxs, q, g, rtol=1e-9)
    for m, ctx in enumerate(ctxs):
        ref = ctx.solve(q[m], g[m], precision=pkg.PRECISION_FP64, rtol=1e-12)
        rel = np.abs(out["signal"][m] - ref["signal"]) / np.abs(ref["signal"])
        assert rel.max() <= MIX_RTOL, (m, rel.max())
    for c in ctxs:
        c.close()


def test_colocated_grids_are_deterministic(pkg, lib):
    """Blocks of different meshes on one SM (two blocks per SM) and two contexts
    solving at the same time from two host threads: every run gives bitwise the
    signals of the same solve run alone.  (A block-level decision once read a
    shared flag that one thread could reset before a slow warp had read it; that
    showed only when another grid's blocks shared the SM.)"""
    import threading
    meshes = pkg.meshgen.uneven_meshes(count=4, seed=3, nmin=6, nmax=14, cube=1.5)
    pick = [meshes[1], meshes[3]]
    ctxs, int4 = contexts(pkg, pick + pick)          # two copies of each mesh
    rng = np.random.default_rng(7)
    q, g, sq = [], [], []
    for cnt in (8, 5):
        d = rng.normal(size=(cnt, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        s = rng.integers(0, 2, size=cnt)
        b = rng.uniform(500, 4000, size=cnt)
        q.append([pkg.sequences.b_to_q(bb, int4[x]) for bb, x in zip(b, s)])
        g.append(d)
        sq.append(s)
    q, g, sq = q + q, g + g, sq + sq
    for c in ctxs:
        c.set_option("mixed.lanes_per_row", 4)
        c.set_option("mixed.blocks_per_sm", 2)
    first = pkg.solve_multi(ctxs[:2], q[:2], g[:2], sq[:2], rtol=1e-9)["signal"]
    for _ in range(3):
        again = pkg.solve_multi(ctxs[:2], q[:2], g[:2], sq[:2], rtol=1e-9)["signal"]
        assert all(np.array_equal(a, b) for a, b in zip(first, again))
    for m in range(2):
        ref = ctxs[m].solve(q[m], g[m], sq[m], precision=pkg.PRECISION_FP64, rtol=1e-12)["signal"]
        assert np.max(np.abs(first[m] - ref) / np.abs(ref)) <= MIX_RTOL
    # two host threads, two contexts of the larger mesh, solving concurrently
    for c in (ctxs[1], ctxs[3]):
        c.set_option("mixed.blocks_per_sm", 1)
    alone = ctxs[1].solve(q[1], g[1], sq[1], precision=pkg.PRECISION_MIXED, rtol=1e-9)["signal"]
    results, errors = {1: [], 3: []}, []

    def work(i):
        try:
            for _ in range(3):
                results[i].append(ctxs[i].solve(q[i], g[i], sq[i], precision=pkg.PRECISION_MIXED, rtol=1e-9)["signal"])
        except Exception as e:          # reported below, after both threads ended
            errors.append(e)

    th = [threading.Thread(target=work, args=(i,)) for i in (1, 3)]
    [t.start() for t in th]
    [t.join() for t in th]
    assert not errors, errors
    assert all(np.array_equal(r, alone) for i in (1, 3) for r in results[i])
    for c in ctxs:
        c.close()
