"""GPU: the batched mixed-precision path (FP32 inner COCG, double-float
residuals) against the FP64 path and the oracle fixtures.  Tolerance: 1e-6
relative signal error (the accuracy the mixed path is specified for)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIX_RTOL = 1e-6


def ctx_for(pkg, w):
    nr = w["n_regions"]
    rc = None if w["multiple"] else np.zeros(nr, np.int32)
    ctx = pkg.Context(0)
    ctx.mesh_upload(w["xyz"], w["tets"], w["region"], nr, rc)
    ctx.set_coefficients(w["D"], w["invT2"], w["kappa"])
    ctx.assemble()
    fns, fos = zip(*[pkg.sequences.profile_samples(p, w["dt"]) for p in w["profiles"]])
    ctx.set_schedule(np.array(fns), np.array(fos), w["dt"])
    return ctx


def signals_of(pkg, w, idx):
    int4 = [p.int4gb() for p in w["profiles"]]
    sel = [w["signals"][i] for i in idx]
    q = np.array([pkg.sequences.b_to_q(b, int4[pi]) for b, _, pi in sel])
    g = np.array([gd for _, gd, _ in sel], float)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    return q, g, np.array([pi for _, _, pi in sel], np.int32)


def test_mixed_matches_golden(pkg, lib, golden):
    for case in golden["cases"]:
        w = pkg.meshgen.workload(case["workload"], seed=case["seed"], n=case["n"])
        ctx = ctx_for(pkg, w)
        sig = case["signals"]
        q = [s["q"] for s in sig]
        g = [s["gdir"] for s in sig]
        pidx = [s["profile"] for s in sig]
        out = ctx.solve(q, g, pidx, precision=pkg.PRECISION_MIXED, rtol=1e-9, max_iterations=2000,
                        compartments=True)
        for k, s in enumerate(sig):
            got = out["signal"][k] / out["S0"]
            rel = abs(got - s["normalized"]) / abs(s["normalized"])
            assert rel <= MIX_RTOL, (case["workload"], case["n"], s["index"], got, s["normalized"], rel)
        ctx.close()


@pytest.mark.parametrize("nsig", [1, 2, 7, 130])
def test_mixed_batches_match_fp64(pkg, lib, nsig):
    """Batches of several sizes (1 to 130 signals: several RHS chunks and
    padding) agree with the FP64 path signal by signal."""
    w = pkg.meshgen.workload("cfg3", n=12)
    ctx = ctx_for(pkg, w)
    idx = np.linspace(0, len(w["signals"]) - 1, nsig).astype(int)
    q, g, pidx = signals_of(pkg, w, idx)
    mixed = ctx.solve(q, g, pidx, precision=pkg.PRECISION_MIXED, rtol=1e-9, compartments=True)
    fp64 = ctx.solve(q, g, pidx, precision=pkg.PRECISION_FP64, rtol=1e-12, compartments=True)
    rel = np.abs(mixed["signal"] - fp64["signal"]) / np.abs(fp64["signal"])
    assert rel.max() <= MIX_RTOL, rel.max()
    assert np.allclose(mixed["compartments"], fp64["compartments"], rtol=1e-5, atol=1e-6 * abs(fp64["signal"]).max())
    ctx.close()


def test_mixed_deterministic_and_solution(pkg, lib):
    w = pkg.meshgen.workload("cfg4", n=10)
    ctx = ctx_for(pkg, w)
    q, g, pidx = signals_of(pkg, w, range(0, 120, 9))
    a = ctx.solve(q, g, pidx, precision=pkg.PRECISION_MIXED, rtol=1e-9)
    ua = ctx.solution(3)
    b = ctx.solve(q, g, pidx, precision=pkg.PRECISION_MIXED, rtol=1e-9)
    ub = ctx.solution(3)
    assert np.array_equal(a["signal"], b["signal"]) and np.array_equal(ua, ub)
    ref = ctx.solve(q, g, pidx, precision=pkg.PRECISION_FP64, rtol=1e-12)
    u64 = ctx.solution(3)
    assert np.max(np.abs(ua - u64)) <= 1e-6 * np.max(np.abs(u64))
    assert np.max(np.abs(a["signal"] - ref["signal"]) / np.abs(ref["signal"])) <= MIX_RTOL
    ctx.close()


def test_mixed_b0_is_one(pkg, lib):
    w = pkg.meshgen.workload("cfg2", n=8)
    ctx = ctx_for(pkg, w)
    out = ctx.solve([0.0, 0.0, 0.0], [[1, 0, 0]] * 3, precision=pkg.PRECISION_MIXED, rtol=1e-9)
    assert np.all(np.abs(out["signal"] / out["S0"] - 1.0) < 1e-9)
    ctx.close()


@pytest.mark.parametrize("nsig", [2, 40])
def test_single_and_two_reduction_iterations_agree(pkg, lib, nsig):
    """The single-reduction inner iteration (default) and the two-reduction one
    ("mixed.inner_reductions" = 2) solve the same problem: both within the
    mixed tolerance of the FP64 path, and both deterministic."""
    w = pkg.meshgen.workload("cfg3", n=14)
    ctx = ctx_for(pkg, w)
    idx = np.linspace(0, len(w["signals"]) - 1, nsig).astype(int)
    q, g, pidx = signals_of(pkg, w, idx)
    fp64 = ctx.solve(q, g, pidx, precision=pkg.PRECISION_FP64, rtol=1e-12)["signal"]
    got = {}
    for mode in (1, 2):
        ctx.set_option("mixed.inner_reductions", mode)
        a = ctx.solve(q, g, pidx, precision=pkg.PRECISION_MIXED, rtol=1e-9)
        b = ctx.solve(q, g, pidx, precision=pkg.PRECISION_MIXED, rtol=1e-9)
        assert np.array_equal(a["signal"], b["signal"]), mode
        rel = np.abs(a["signal"] - fp64) / np.abs(fp64)
        assert rel.max() <= MIX_RTOL, (mode, rel.max())
        got[mode] = a
    # both forms do comparable work (inner iterations within a factor of 1.5)
    it1, it2 = got[1]["stats"]["total_iterations"], got[2]["stats"]["total_iterations"]
    assert 0.66 * it2 <= it1 <= 1.5 * it2, (it1, it2)
    ctx.close()
