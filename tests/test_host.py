"""Host-side logic of the package (no GPU): sequences, meshes, API plumbing."""

import numpy as np
import pytest

import oracle


def test_mesh_matches_oracle(pkg):
    for n in (3, 5):
        a = pkg.meshgen.kuhn_box(-2.5, 2.5, n)
        b = oracle.box_mesh((-2.5,) * 3, (2.5,) * 3, n)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("name", ["pgse", "cos_ogse"])
def test_profiles_match_oracle(pkg, name):
    P = getattr(pkg.sequences, name)(10600, 43100)
    O = oracle.PGSE(10600, 43100) if name == "pgse" else oracle.CosOGSE(10600, 43100)
    assert abs(P.int4gb() / O.int4gb() - 1) < 1e-13
    fn, fo = pkg.sequences.profile_samples(P, 200.0)
    tn, to = oracle.reference_schedule(O.T, 200.0)
    assert np.array_equal(fn, [O.f(t) for t in tn]) and np.array_equal(fo, [O.f(t) for t in to])
    for t in (0.0, 5000.0, 10600.0, 20000.0, 43100.0, 50000.0, 53700.0):
        assert abs(P.F(t) - O.F(t)) < 1e-9


def test_other_profiles_echo(pkg):
    # F(T) = 0 (echo condition) for every built-in profile
    for p in (pkg.sequences.double_pgse(5000, 20000), pkg.sequences.sin_ogse(10600, 43100),
              pkg.sequences.trapezoid_pgse(10600, 43100), pkg.sequences.pgse(1000, 5000, t0=100, seq_ext=100)):
        assert abs(p.F(p.T)) < 1e-6 * p.T
        assert p.int4gb() > 0


def test_trapezoid_int4gb_against_sympy(pkg):
    sp = pytest.importorskip("sympy")
    s, u = sp.Symbol("s"), sp.Symbol("u")
    d, D = 10600.0, 43100.0
    Dd, tau, t0 = d + D, d / 3.0, 0.0
    fs = sp.Piecewise((0., s < t0), ((s - t0) / tau, s < tau + t0), (1., s < d - tau + t0),
                      (-(s - t0 - d) / tau, s < d + t0), (0., s < D + t0), (-(s - t0 - D) / tau, s < D + tau + t0),
                      (-1., s < Dd - tau + t0), ((s - t0 - Dd) / tau, s < Dd + t0), (0., True))
    ifs = sp.integrate(fs.subs(s, u), (u, 0, s))
    ref = float(sp.integrate(ifs * ifs, (s, 0, Dd)))
    # sympy works in 15-digit Floats here (tau = delta/3 is inexact); agree to 1e-10
    assert abs(pkg.sequences.trapezoid_pgse(d, D).int4gb() / ref - 1) < 1e-10


def test_q_conversions(pkg):
    p = pkg.sequences.pgse(1000, 10000)
    q = pkg.sequences.b_to_q(1000.0, p.int4gb())
    assert "%.3e" % q == "3.216e-04" and "%.3f" % pkg.sequences.q_to_g(q) == "1.202"
    assert abs(pkg.sequences.q_to_b(q, p.int4gb()) - 1000.0) < 1e-9


def test_mri_parameters_flow(pkg):
    para = pkg.MRI_parameters()
    para.bvalue = 1000
    para.delta, para.Delta = 10600, 43100
    mesh = pkg.Mesh(*pkg.meshgen.kuhn_box(-1, 1, 2))
    para.set_gradient_dir(mesh, 0, 2, 0)
    assert np.allclose(para.gdir, [0, 1, 0])
    para.Apply()
    assert para.T == 53700.0 and para.qvalue > 0
    with pytest.raises(ValueError):
        para.set_gradient_dir(mesh, 0, 0, 0)


def test_sympy_profile_matches(pkg):
    sp = pytest.importorskip("sympy")
    para = pkg.MRI_parameters()
    para.bvalue = 1000
    para.T = 53700.0
    s = para.s
    para.fs_sym = sp.Piecewise((1., s < 10600.), (0., s < 43100.), (-1., s < 53700.), (0., True))
    para.Apply()
    q2 = pkg.sequences.b_to_q(1000.0, pkg.sequences.pgse(10600, 43100).int4gb())
    assert abs(para.qvalue / q2 - 1) < 1e-14
    assert para.time_profile(10600.0) == 0.0 and para.time_profile(200.0) == 1.0


def test_strong_periodic_accepted_and_integral_schedule(pkg):
    """IsDomainPeriodic = True with PeriodicDir set selects the strong form
    (Apply accepts it); its schedule is ift at both levels, with
    F_new[s] = F_old[s + 1] (tp of a step is t of the one before)."""
    mesh = pkg.Mesh(*pkg.meshgen.kuhn_box(-1, 1, 2))
    para = pkg.MRI_parameters()
    dom = pkg.MyDomain(mesh, para)
    dom.PeriodicDir = [1, 0, 0]
    dom.IsDomainPeriodic = True
    dom.Apply()
    p = pkg.sequences.pgse(1000.0, 3000.0)
    Fn, Fo = pkg.sequences.integral_samples(p, 200.0)
    assert len(Fn) == len(Fo) and np.allclose(Fn[:-1], Fo[1:])
    # the reference's first solve has t = tp = 0 (DmriFemLib.py:889-905)
    assert Fo[0] == 0.0 and Fn[0] == 0.0 and np.isclose(Fn[1], p.F(200.0))
    assert np.allclose(Fo, pkg.sequences.phase_samples(p, 200.0))


def test_phase_samples(pkg):
    """F(tp) on the explicit level: F(0) at the first step, then F((n-1) k)."""
    p = pkg.sequences.pgse(1000.0, 3000.0)
    F = pkg.sequences.phase_samples(p, 200.0)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    assert len(F) == len(fo) and F[0] == 0.0
    assert abs(F[1] - p.F(0.0)) < 1e-15 and abs(F[2] - p.F(200.0)) < 1e-12
    assert abs(F[-1] - p.F((len(F) - 2) * 200.0)) < 1e-9


def test_domain_regions(pkg):
    xyz, tets = pkg.meshgen.kuhn_box(-5, 5, 4)
    reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0, 0)], [3.0])
    mesh = pkg.Mesh(xyz, tets)
    dom = pkg.MyDomain(mesh, pkg.MRI_parameters())
    dom.IsDomainMultiple = True
    dom.phase = reg.astype(float)
    r, nr, rc = dom.regions()
    assert nr == 2 and np.array_equal(r, reg) and list(rc) == [0, 1]
    dom.IsDomainMultiple = False
    r, nr, rc = dom.regions()
    assert nr == 1 and not r.any()


def test_workloads_shapes(pkg):
    w = pkg.meshgen.workload("cfg3", n=8)
    assert len(w["signals"]) == 512 and len(w["profiles"]) == 2
    cs, rs = w["cylinders"]
    assert len(cs) == 8
    for i in range(8):
        for j in range(i):
            assert np.hypot(*(cs[i] - cs[j])) > rs[i] + rs[j]
    w4 = pkg.meshgen.workload("cfg4", n=8)
    assert len(w4["signals"]) == 120 and set(np.unique(w4["region"])) <= {0, 1, 2, 3}
    d = pkg.meshgen.fibonacci_directions(64)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0)


def test_projection_of_cell_values(pkg):
    """P1 projection: constants are reproduced and M x = b holds."""
    xyz, tets = pkg.meshgen.kuhn_box(-3, 3, 5)
    m = pkg.Mesh(xyz, tets)
    x = pkg.project_cell_values(m, np.full(len(tets), 2.5))
    assert np.max(np.abs(x - 2.5)) < 1e-12
    rng = np.random.default_rng(2)
    v = rng.uniform(0.0, 1.0, len(tets))
    x = pkg.project_cell_values(m, v)
    sd = oracle.duplicated_system(xyz, tets, np.zeros(len(tets), np.int64), 3e-3)
    M = sd["M"]                                # one compartment: dofs are vertices in order
    assert np.array_equal(sd["vertex"], np.arange(len(xyz)))
    vol, _, _ = oracle.element_geometry(xyz, tets)
    b = np.bincount(tets.ravel(), weights=np.repeat(v * vol / 4.0, 4), minlength=len(xyz))
    assert np.max(np.abs(M @ x - b)) <= 1e-12 * np.max(np.abs(b))
