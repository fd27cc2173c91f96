"""GPU: strong pseudo-periodic form (bt_set_periodic_mode(BT_PERIODIC_STRONG)) against
the CPU oracle's folded complex system (FP64, 1e-9), the closed form of the
homogeneous box, the reference-named API, and the refusals."""

import numpy as np
import pytest

import oracle
from oracle import strong

pytestmark = pytest.mark.gpu

SIG_RTOL = 1e-9
DELTA, BIGDELTA, DT = 2000.0, 5000.0, 100.0


def cube_cylinder_regions(xyz, tets, r):
    """z-cylinder on whole Kuhn cubes (the staircase is the same on opposite faces)."""
    X = xyz[tets]
    c = 0.5 * (X.min(axis=1) + X.max(axis=1))
    return (c[:, 0] ** 2 + c[:, 1] ** 2 < r * r).astype(np.int32)


def strong_ctx(pkg, xyz, tets, reg, nr, D, iT2, kp, pdir, seq, dt=DT):
    ctx = pkg.Context(0)
    ctx.mesh_upload(xyz, tets, reg, nr)
    ctx.set_coefficients(D, iT2, kp)
    ctx.assemble()
    ctx.set_periodic_mode("strong")
    ctx.set_periodic(pdir)
    fn, fo = pkg.sequences.profile_samples(seq, dt)
    ctx.set_schedule(fn, fo, dt)
    ctx.set_schedule_integral(*pkg.sequences.integral_samples(seq, dt))
    return ctx


def test_homogeneous_box_closed_form(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(0.0, 6.0, 6)
    reg = np.zeros(len(tets), np.int32)
    seq = pkg.sequences.pgse(DELTA, BIGDELTA)
    q = pkg.sequences.b_to_q(3000.0, seq.int4gb())
    D, iT2 = 2e-3, 1.0 / 8e4
    ctx = strong_ctx(pkg, xyz, tets, reg, 1, [D], [iT2], None, [1, 0, 0], seq)
    out = ctx.solve([q], [1.0, 0.0, 0.0], rtol=1e-13, max_iterations=5000)
    exact = strong.uniform_box_signal(216.0, D, iT2, oracle.PGSE(DELTA, BIGDELTA), q, DT)
    assert abs(out["signal"][0] - exact) <= 1e-10 * abs(exact), (out["signal"][0], exact)
    info = ctx.strong_periodic_info()
    # 7^3 vertices, the x = 6 face folded onto x = 0
    assert info["n_classes"] == 6 * 7 * 7 and info["n_dofs"] == 6 * 7 * 7
    u = ctx.solution(0)
    assert np.max(np.abs(u - u[0])) <= 1e-11 * abs(u[0])
    ctx.close()


@pytest.mark.parametrize("pdir,g", [([1, 1, 1], (1.0, 0.4, 0.3)), ([1, 1, 0], (0.6, 1.0, 0.0)),
                                    ([0, 1, 0], (0.2, 1.0, 0.0))])
def test_two_compartments_match_oracle(pkg, lib, pdir, g):
    xyz, tets = pkg.meshgen.kuhn_box(-5.0, 5.0, 8)
    reg = cube_cylinder_regions(xyz, tets, 2.6)
    D = [3e-3, 1.5e-3]
    iT2 = [0.0, 1.0 / 6e4]
    kp = np.array([[0.0, 2e-5], [2e-5, 0.0]])
    seq = pkg.sequences.pgse(DELTA, BIGDELTA)
    g = np.asarray(g) / np.linalg.norm(g)
    qs = [pkg.sequences.b_to_q(b, seq.int4gb()) for b in (1000.0, 2500.0)]
    ctx = strong_ctx(pkg, xyz, tets, reg, 2, D, iT2, kp, pdir, seq)
    out = ctx.solve(qs, np.tile(g, (2, 1)), rtol=1e-13, max_iterations=5000, compartments=True)
    sd = strong.duplicated_strong(xyz, tets, reg, np.array(D), np.array(iT2), kp, pdir, g)
    for i, q in enumerate(qs):
        ref = strong.solve_strong(sd, oracle.PGSE(DELTA, BIGDELTA), q, DT)
        assert abs(out["signal"][i] - ref["signal"]) <= SIG_RTOL * abs(ref["signal"]), (out["signal"][i], ref["signal"])
        assert np.allclose(out["compartments"][i], ref["compartments"], rtol=1e-9, atol=1e-9 * abs(ref["signal"]))
        assert len(ctx.solution(i)) == ctx.info()["n_dofs"]     # unfolded dofs
    info = ctx.strong_periodic_info()
    assert info["n_dofs"] == sd["n"]
    ctx.close()


def test_solution_on_unfolded_dofs(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(-5.0, 5.0, 6)
    reg = cube_cylinder_regions(xyz, tets, 2.6)
    seq = pkg.sequences.pgse(DELTA, BIGDELTA)
    q = pkg.sequences.b_to_q(2000.0, seq.int4gb())
    g = np.array([0.8, 0.6, 0.0])
    ctx = strong_ctx(pkg, xyz, tets, reg, 2, [3e-3, 3e-3], None, np.array([[0, 1e-5], [1e-5, 0]]), [1, 1, 1], seq)
    ctx.solve([q], g, rtol=1e-13, max_iterations=5000)
    u = ctx.solution(0)
    sd = strong.duplicated_strong(xyz, tets, reg, 3e-3, 0.0, np.array([[0, 1e-5], [1e-5, 0]]), [1, 1, 1], g)
    ref = strong.solve_strong(sd, oracle.PGSE(DELTA, BIGDELTA), q, DT)
    # unfolded dof (vertex v, compartment c) -> oracle dof of (class of v, c)
    plain = oracle.duplicated_system(xyz, tets, reg, 3e-3)
    cls = sd["class_of_vertex"][plain["vertex"]]
    od = sd["dof"][cls, plain["field"]]
    assert np.all(od >= 0)
    assert np.max(np.abs(u - ref["u"][od])) <= 1e-9 * np.max(np.abs(ref["u"]))
    ctx.close()


def test_refusals(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(-5.0, 5.0, 6)
    seq = pkg.sequences.pgse(DELTA, BIGDELTA)
    q = pkg.sequences.b_to_q(1000.0, seq.int4gb())
    # a gradient with a component normal to the non-periodic faces where the
    # cylinder's interface meets them
    reg = cube_cylinder_regions(xyz, tets, 2.6)
    ctx = strong_ctx(pkg, xyz, tets, reg, 2, [3e-3, 3e-3], None, 1e-5, [1, 1, 0], seq)
    with pytest.raises(RuntimeError, match="must vanish"):
        ctx.solve([q], [0.3, 0.2, 1.0], rtol=1e-12, max_iterations=5000)
    ctx.solve([q], [0.6, 0.8, 0.0], rtol=1e-12, max_iterations=5000)          # in-plane: accepted
    with pytest.raises(RuntimeError, match="FP64"):
        ctx.solve([q], [0.6, 0.8, 0.0], precision=pkg.PRECISION_MIXED, rtol=1e-9, max_iterations=5000)
    with pytest.raises(RuntimeError, match="strong"):
        ctx.adjoint(q, [0.6, 0.8, 0.0])
    # weak mode again: the same directions, the penalty form
    ctx.set_periodic_mode("weak")
    assert ctx.periodic_info()["active"] == 1 and ctx.strong_periodic_info()["n_dofs"] == 0
    ctx.close()
    # compartments that differ across a periodic face (per-tetrahedron staircase)
    reg2 = pkg.meshgen.cylinder_regions(xyz, tets, [(0.0, 0.0)], [2.6])
    ctx = strong_ctx(pkg, xyz, tets, reg2, 2, [3e-3, 3e-3], None, 1e-5, [0, 0, 1], seq)
    with pytest.raises(RuntimeError, match="not periodic"):
        ctx.solve([q], [0.0, 0.0, 1.0], rtol=1e-12, max_iterations=5000)
    ctx.close()
    # a mesh whose max face has no matching vertices
    xyz3 = xyz.copy()
    on_max = np.isclose(xyz3[:, 0], 5.0) & ~np.isclose(xyz3[:, 1], -5.0) & ~np.isclose(xyz3[:, 1], 5.0)
    xyz3[on_max, 1] += 0.3 * (10.0 / 6)
    ctx = strong_ctx(pkg, xyz3, tets, np.zeros(len(tets), np.int32), 1, [3e-3], None, None, [1, 0, 0], seq)
    with pytest.raises(RuntimeError, match="mesh not periodic"):
        ctx.solve([q], [1.0, 0.0, 0.0], rtol=1e-12, max_iterations=5000)
    ctx.close()


def test_reference_api(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(-5.0, 5.0, 6)
    reg = cube_cylinder_regions(xyz, tets, 2.6)
    mesh = pkg.Mesh(xyz, tets, reg)
    para = pkg.MRI_parameters()
    para.bvalue, para.delta, para.Delta = 2000.0, DELTA, BIGDELTA
    para.set_gradient_dir(mesh, 1, 1, 0)
    para.Apply()
    dom = pkg.MyDomain(mesh, para)
    dom.PeriodicDir = [1, 1, 1]
    dom.IsDomainPeriodic = True
    dom.IsDomainMultiple = True
    dom.kappa = 1e-5
    dom.Apply()
    dom.D = 3e-3
    sim = pkg.MRI_simulation()
    sim.k = DT
    s = sim.solve(dom, para)
    g = np.array([1.0, 1.0, 0.0]) / np.sqrt(2.0)
    sd = strong.duplicated_strong(xyz, tets, reg, 3e-3, 0.0, 1e-5, [1, 1, 1], g)
    ref = strong.solve_strong(sd, oracle.PGSE(DELTA, BIGDELTA), para.qvalue, DT)
    assert abs(s - ref["signal"]) <= SIG_RTOL * abs(ref["signal"])
    # the weak form on the same domain gives another signal
    dom.IsDomainPeriodic = False
    dom.Apply()
    w = sim.solve(dom, para)
    assert abs(w - s) > 1e-6 * abs(s)


def test_full_schedule_matches_golden(pkg, lib):
    """270 steps on the 12^3 periodic box of tests/golden/oracle_strong_signals.json
    (made by tests/golden/make_strong_fixture.py from the oracle)."""
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "oracle_strong_signals.json")) as fh:
        gold = json.load(fh)
    s = gold["setup"]
    lo, hi = s["box"]
    xyz, tets = pkg.meshgen.kuhn_box(lo, hi, s["cubes_per_axis"])
    reg = cube_cylinder_regions(xyz, tets, s["radius"])
    seq = pkg.sequences.pgse(s["delta"], s["Delta"])
    kp = np.array([[0.0, s["kappa"]], [s["kappa"], 0.0]])
    ctx = strong_ctx(pkg, xyz, tets, reg, 2, s["D"], None, kp, s["periodic_dir"], seq, s["dt"])
    q = [g["q"] for g in gold["signals"]]
    gd = [np.asarray(g["g"]) / np.linalg.norm(g["g"]) for g in gold["signals"]]
    out = ctx.solve(q, gd, rtol=1e-13, max_iterations=20000, compartments=True)
    assert ctx.strong_periodic_info()["n_dofs"] == gold["n_dofs"]
    for i, g in enumerate(gold["signals"]):
        assert abs(out["signal"][i] - g["signal"]) <= SIG_RTOL * abs(g["signal"]), (i, out["signal"][i], g["signal"])
        assert np.allclose(out["compartments"][i], g["compartments"], rtol=1e-9)
    ctx.close()


def test_anisotropic_tensor_t2_field_and_initial_condition(pkg, lib):
    """Per-cell anisotropic D tensor, per-cell T2 and a non-uniform initial
    condition through the strong form, against the oracle (which takes the
    same per-cell tensor in its first-order, M_D and boundary terms).  The
    fields vary per cube column (x, y) only, so they are periodic across the
    z faces, where the cylinder's interface meets the boundary (a field that
    differs across a periodic face is refused, as the literal form's
    phase-blind outer term would not cancel there)."""
    xyz, tets = pkg.meshgen.kuhn_box(-5.0, 5.0, 6)
    reg = cube_cylinder_regions(xyz, tets, 2.6)
    rng = np.random.default_rng(11)
    n_t = len(tets)
    X = xyz[tets].min(axis=1)
    col = (np.rint((X[:, 0] + 5.0) / (10.0 / 6)) * 6 + np.rint((X[:, 1] + 5.0) / (10.0 / 6))).astype(int)
    base = np.where(reg == 1, 1.5e-3, 3e-3)
    r3, o3, rt = rng.random((36, 3)), rng.random((36, 3)), rng.random(36)
    D6 = np.zeros((n_t, 6))
    D6[:, :3] = base[:, None] * (1.0 + 0.4 * r3[col])
    D6[:, 3:] = base[:, None] * 0.15 * (o3[col] - 0.5)
    iT = 1.0 / (5e4 + 5e4 * rt[col])
    u0 = 1.0 + 0.2 * np.cos(2 * np.pi * xyz[:, 0] / 10.0)       # periodic along x
    seq = pkg.sequences.pgse(DELTA, BIGDELTA)
    q = pkg.sequences.b_to_q(2000.0, seq.int4gb())
    g = np.array([0.6, 0.8, 0.0])
    kp = np.array([[0.0, 1e-5], [1e-5, 0.0]])
    ctx = pkg.Context(0)
    ctx.mesh_upload(xyz, tets, reg, 2)
    ctx.set_coefficients([3e-3, 1.5e-3], None, kp)
    ctx.set_cell_diffusion(D6)
    ctx.set_cell_T2(iT)
    ctx.assemble()
    ctx.set_periodic_mode("strong")
    ctx.set_periodic([1, 1, 1])
    fn, fo = pkg.sequences.profile_samples(seq, DT)
    ctx.set_schedule(fn, fo, DT)
    ctx.set_schedule_integral(*pkg.sequences.integral_samples(seq, DT))
    out = ctx.solve([q], g, u0=u0, rtol=1e-13, max_iterations=5000)
    Dt = np.zeros((n_t, 3, 3))
    for k, (a, b) in enumerate([(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]):
        Dt[:, a, b] = D6[:, k]
        Dt[:, b, a] = D6[:, k]
    sd = strong.duplicated_strong(xyz, tets, reg, Dt, iT, kp, [1, 1, 1], g)
    ref = strong.solve_strong(sd, oracle.PGSE(DELTA, BIGDELTA), q, DT, u0=u0)
    assert abs(out["signal"][0] - ref["signal"]) <= SIG_RTOL * abs(ref["signal"]), (out["signal"][0], ref["signal"])
    ctx.close()


def test_batched_stepper_matches_single(pkg, lib):
    """Signals share the batched strong stepper (one lane each, its own direction);
    the same signals one launch each give the same values (1e-10), and outputs
    keep the call's order."""
    xyz, tets = pkg.meshgen.kuhn_box(-5.0, 5.0, 6)
    reg = cube_cylinder_regions(xyz, tets, 2.6)
    seq = pkg.sequences.pgse(DELTA, BIGDELTA)
    kp = np.array([[0.0, 2e-5], [2e-5, 0.0]])
    ctx = strong_ctx(pkg, xyz, tets, reg, 2, [3e-3, 1.5e-3], [0.0, 1.0 / 6e4], kp, [1, 1, 1], seq)
    bs = [500.0, 1000.0, 1500.0, 2000.0, 2500.0, 3000.0]
    g1, g2 = np.array([1.0, 0.4, 0.3]), np.array([0.2, 0.5, 1.0])
    q = np.array([pkg.sequences.b_to_q(b, seq.int4gb()) for b in bs] * 2
                 + [pkg.sequences.b_to_q(2200.0, seq.int4gb())] * 30)
    rng = np.random.default_rng(2)
    g3 = rng.normal(size=(30, 3))                                # 30 more directions: 42 signals, two launches
    g = np.concatenate([np.array([g1] * 6 + [g2] * 6), g3 / np.linalg.norm(g3, axis=1)[:, None]])
    perm = rng.permutation(42)                                   # interleaved in the call
    q, g = q[perm], g[perm]
    ctx.set_option("strong.batch", 1)
    a = ctx.solve(q, g, rtol=1e-13, max_iterations=5000, compartments=True)
    ua = [ctx.solution(i) for i in (0, 5, 41)]
    ctx.set_option("strong.batch", 0)
    b = ctx.solve(q, g, rtol=1e-13, max_iterations=5000, compartments=True)
    assert np.max(np.abs(a["signal"] - b["signal"]) / np.abs(b["signal"])) <= 1e-10
    assert np.allclose(a["compartments"], b["compartments"], rtol=1e-10, atol=1e-12)
    for i, u in zip((0, 5, 41), ua):
        ub = ctx.solution(i)
        assert np.max(np.abs(u - ub)) <= 1e-10 * np.max(np.abs(ub))
    # a b-series of one direction (the launch reads its direction terms precombined)
    qs = np.array([pkg.sequences.b_to_q(b, seq.int4gb()) for b in np.linspace(500.0, 4000.0, 8)])
    gs = np.tile(g2 / np.linalg.norm(g2), (8, 1))
    ctx.set_option("strong.batch", 1)
    a = ctx.solve(qs, gs, rtol=1e-13, max_iterations=5000)
    ctx.set_option("strong.batch", 0)
    b = ctx.solve(qs, gs, rtol=1e-13, max_iterations=5000)
    assert np.max(np.abs(a["signal"] - b["signal"]) / np.abs(b["signal"])) <= 1e-10
    ctx.close()


def test_batched_stepper_groups_sequences(pkg, lib):
    """Two sequences (PGSE and cos-OGSE of the same length) interleaved in one
    call: the batched launches group by sequence, every signal matches its
    single launch (1e-10) in the call's order."""
    xyz, tets = pkg.meshgen.kuhn_box(-5.0, 5.0, 6)
    reg = cube_cylinder_regions(xyz, tets, 2.6)
    seqs = [pkg.sequences.pgse(DELTA, BIGDELTA), pkg.sequences.cos_ogse(DELTA, BIGDELTA)]
    ctx = pkg.Context(0)
    ctx.mesh_upload(xyz, tets, reg, 2)
    ctx.set_coefficients([3e-3, 2e-3], None, np.array([[0.0, 1e-5], [1e-5, 0.0]]))
    ctx.assemble()
    ctx.set_periodic_mode("strong")
    ctx.set_periodic([1, 1, 1])
    fns, fos = zip(*[pkg.sequences.profile_samples(sq, DT) for sq in seqs])
    ctx.set_schedule(np.array(fns), np.array(fos), DT)
    Fs = [pkg.sequences.integral_samples(sq, DT) for sq in seqs]
    ctx.set_schedule_integral(np.array([f[0] for f in Fs]), np.array([f[1] for f in Fs]))
    rng = np.random.default_rng(7)
    n = 10
    sq = rng.integers(0, 2, n).astype(np.int32)
    g = rng.normal(size=(n, 3))
    g /= np.linalg.norm(g, axis=1)[:, None]
    q = np.array([pkg.sequences.b_to_q(b, seqs[s].int4gb()) for b, s in zip(np.linspace(500.0, 3000.0, n), sq)])
    ctx.set_option("strong.batch", 1)
    a = ctx.solve(q, g, sq, rtol=1e-13, max_iterations=5000)
    ctx.set_option("strong.batch", 0)
    b = ctx.solve(q, g, sq, rtol=1e-13, max_iterations=5000)
    assert np.max(np.abs(a["signal"] - b["signal"]) / np.abs(b["signal"])) <= 1e-10
    ctx.close()
