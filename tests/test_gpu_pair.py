"""GPU: the FP64 path's two-signals-a-launch stepper (k_step64_pair, option
fp64.pair_signals) against the one-signal-a-launch stepper (k_step64) and the
oracle fixtures.

Both kernels do a signal's per-row arithmetic in the same order; with the same
grid the block partial sums are the same, so the signals agree to rounding
(tolerance 1e-12 relative; the FP64 path's own bar against the oracle is
1e-9).  A pair's two signals converge separately: each keeps its own COCG
scalars and stopping test, so the iteration counts are the single kernel's."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PAIR_RTOL = 1e-12


def _ctx(pkg, w):
    nr = w["n_regions"]
    rc = None if w["multiple"] else np.zeros(nr, np.int32)
    ctx = pkg.Context(0)
    ctx.mesh_upload(w["xyz"], w["tets"], w["region"], nr, rc)
    ctx.set_coefficients(w["D"], w["invT2"], w["kappa"])
    ctx.assemble()
    fns, fos = zip(*[pkg.sequences.profile_samples(p, w["dt"]) for p in w["profiles"]])
    ctx.set_schedule(np.array(fns), np.array(fos), w["dt"])
    return ctx


def _signals(pkg, w, idx):
    int4 = [p.int4gb() for p in w["profiles"]]
    sel = [w["signals"][i] for i in idx]
    q = np.array([pkg.sequences.b_to_q(b, int4[pi]) for b, _, pi in sel])
    g = np.array([gd for _, gd, _ in sel], float)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    return q, g, np.array([pi for _, _, pi in sel], np.int32)


def _run(ctx, mode, q, g, seq, u0=None):
    ctx.set_option("fp64.pair_signals", mode)
    out = ctx.solve(q, g, seq, u0=u0, rtol=1e-12, max_iterations=5000, compartments=True)
    sols = [ctx.solution(k) for k in range(len(q))]
    its = ctx.iterations(len(q), out["stats"]["steps"])
    return out, sols, its


@pytest.mark.parametrize("mode", [1, 2])
def test_pair_matches_single_launches(pkg, lib, mode):
    """Five signals: a pair of one direction and two sequences, a signal of
    another direction (breaks the pairing), then a pair of b = 0 and b > 0
    (one converges long before the other)."""
    w = pkg.meshgen.workload("cfg3", n=10)
    ctx = _ctx(pkg, w)
    q, g, seq = _signals(pkg, w, [0, 1, 2, 3, 4])
    g[1] = g[0]
    g[3] = g[4] = g[2] * -1.0
    seq[0], seq[1] = 0, len(w["profiles"]) - 1
    q[3] = 0.0
    ref, ref_u, ref_it = _run(ctx, 0, q, g, seq)
    got, got_u, got_it = _run(ctx, mode, q, g, seq)
    ctx.set_option("fp64.pair_signals", 1)
    assert got["stats"]["kernel_launches"] == 5 + 3 + 5
    assert ref["stats"]["kernel_launches"] == 3 * 5
    rel = np.abs(got["signal"] - ref["signal"]) / np.abs(ref["signal"])
    assert rel.max() <= PAIR_RTOL, rel
    assert np.allclose(got["compartments"], ref["compartments"], rtol=PAIR_RTOL, atol=PAIR_RTOL * abs(ref["S0"]))
    for k in range(len(q)):
        err = np.abs(got_u[k] - ref_u[k]).max() / np.abs(ref_u[k]).max()
        assert err <= 1e-11, (k, err)
    assert abs(got["signal"][3] / got["S0"] - 1.0) <= 1e-12    # b = 0 keeps the signal
    # same stopping test per signal: iteration counts equal up to the rounding of the sums
    assert np.abs(got_it - ref_it).max() <= 1, np.abs(got_it - ref_it).max()
    assert abs(int(got_it.sum()) - int(ref_it.sum())) <= 0.01 * int(ref_it.sum())
    ctx.close()


def test_pair_interleaved_directions(pkg, lib):
    """Directions A, B, A, B, A: signals 0 and 2, 1 and 3 are paired across the
    positions (4 runs alone); outputs stay in the call's order."""
    w = pkg.meshgen.workload("cfg3", n=10)
    ctx = _ctx(pkg, w)
    q, g, seq = _signals(pkg, w, [0, 9, 2, 11, 4])
    assert not np.array_equal(g[0], g[1])
    g[2] = g[4] = g[0]
    g[3] = g[1]
    ref, ref_u, ref_it = _run(ctx, 0, q, g, seq)
    got, got_u, got_it = _run(ctx, 2, q, g, seq)
    assert got["stats"]["kernel_launches"] == 5 + 5 + 3
    rel = np.abs(got["signal"] - ref["signal"]) / np.abs(ref["signal"])
    assert rel.max() <= PAIR_RTOL, rel
    for k in range(len(q)):
        err = np.abs(got_u[k] - ref_u[k]).max() / np.abs(ref_u[k]).max()
        assert err <= 1e-11, (k, err)
    assert np.abs(got_it - ref_it).max() <= 1
    ctx.close()


def test_pair_initial_condition_and_golden(pkg, lib, golden):
    """A non-unit initial condition through both forms, and the full-size
    two-compartment fixture through the pair (its signals share a direction)."""
    w = pkg.meshgen.workload("cfg2", n=8)
    ctx = _ctx(pkg, w)
    idx = np.arange(min(4, len(w["signals"])))
    q, g, seq = _signals(pkg, w, idx)
    g[:] = g[0]
    rng = np.random.default_rng(7)
    u0 = 0.5 + rng.random(ctx.n_vertices)
    ref, _, _ = _run(ctx, 0, q, g, seq, u0=u0)
    got, _, _ = _run(ctx, 1, q, g, seq, u0=u0)
    rel = np.abs(got["signal"] - ref["signal"]) / np.abs(ref["signal"])
    assert rel.max() <= PAIR_RTOL, rel
    ctx.close()
    case = next(c for c in golden["cases"] if c["workload"] == "cfg2")
    w = pkg.meshgen.workload(case["workload"], seed=case["seed"], n=case["n"])
    ctx = _ctx(pkg, w)
    sig = case["signals"]
    gd = [s["gdir"] for s in sig]
    assert all(np.array_equal(gd[0], x) for x in gd)
    ctx.set_option("fp64.pair_signals", 1)
    out = ctx.solve([s["q"] for s in sig], gd, [s["profile"] for s in sig], rtol=1e-12, max_iterations=5000)
    assert out["stats"]["kernel_launches"] == 5 * (len(sig) // 2) + 3 * (len(sig) % 2)
    for k, s in enumerate(sig):
        rel = abs(out["signal"][k] / out["S0"] - s["normalized"]) / abs(s["normalized"])
        assert rel <= 1e-9, (s["index"], rel)
    ctx.close()
