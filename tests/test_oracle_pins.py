"""The CPU oracle against the reference's own printed results and exact
identities (no GPU)."""

import math

import numpy as np
import pytest

import oracle
from oracle.sequence import q_to_g


def test_boxmesh_counts():
    # ConvergenceTest.ipynb:261-263: BoxMesh n=5 has 216 points, 750 tetra
    xyz, tets = oracle.box_mesh((-2.5,) * 3, (2.5,) * 3, 5)
    assert len(xyz) == 216 and len(tets) == 750
    vol, _, _ = oracle.element_geometry(xyz, tets)
    assert np.allclose(vol, 1.0 / 6.0) and math.isclose(vol.sum(), 125.0)


def test_convergence_test_kat(kats):
    """Reference printed: q 3.216e-04, g 1.202, Signal 1.055e+02, Normalized
    8.440078e-01, hmin 5.413e-01 (ConvergenceTest.ipynb cell 10)."""
    k = kats["convergence_test_3d_box"]
    s, p = k["setup"], k["printed"]
    n = s["cubes_per_axis"]
    xyz, tets = oracle.box_mesh((s["box"][0],) * 3, (s["box"][1],) * 3, n)
    assert math.isclose(math.sqrt(3.0) * 5.0 / n, p["hmin"], rel_tol=1e-3)
    seq = oracle.PGSE(s["delta"], s["Delta"])
    q = oracle.bvalue_to_q(s["b"], seq.int4gb())
    assert "%.3e" % q == "%.3e" % p["q"]
    assert "%.3f" % q_to_g(q) == "%.3f" % p["g"]
    sd = oracle.duplicated_system(xyz, tets, np.zeros(len(tets), np.int32), s["D"])
    r = oracle.solve_duplicated(sd, seq, q, s["gdir"], s["dt"], loop="lt_T")
    assert r.steps == 1100
    assert "%.6e" % r.normalized == "%.6e" % p["normalized"]      # all 7 printed digits
    assert "%.3e" % r.signal == "%.3e" % p["signal"]
    assert math.isclose(r.S0, p["voi"])


def test_b0_is_one():
    xyz, tets = oracle.box_mesh((-3,) * 3, (3,) * 3, 4)
    reg = oracle.region_from_centroids(xyz, tets, [lambda c: (c ** 2).sum(1) < 4])
    sd = oracle.duplicated_system(xyz, tets, reg, 3e-3, 0.0, 1e-5)
    r = oracle.solve_duplicated(sd, oracle.PGSE(1000, 3000), 0.0, (1, 0, 0), 200.0)
    assert abs(r.normalized - 1.0) < 1e-12


def test_uniform_T2_exact():
    xyz, tets = oracle.box_mesh((-3,) * 3, (3,) * 3, 4)
    T2, k, th = 5e4, 200.0, 0.5
    sd = oracle.duplicated_system(xyz, tets, np.zeros(len(tets), np.int32), 3e-3, 1.0 / T2)
    r = oracle.solve_duplicated(sd, oracle.PGSE(1000, 3000), 0.0, (1, 0, 0), k)
    exact = ((1 - (1 - th) * k / T2) / (1 + th * k / T2)) ** r.steps
    assert abs(r.normalized - exact) < 1e-13


@pytest.mark.parametrize("mode", ["facet", "cr"])
def test_two_field_literal_equals_duplicated(mode):
    xyz, tets = oracle.box_mesh((-10,) * 3, (10,) * 3, 6)
    reg = oracle.region_from_centroids(xyz, tets, [lambda c: c[:, 0] ** 2 + c[:, 1] ** 2 < 36])
    seq = oracle.PGSE(10600, 43100)
    q = oracle.bvalue_to_q(3000, seq.int4gb())
    sd = oracle.duplicated_system(xyz, tets, reg, 3e-3, 0.0, 1e-5, kappa_mode=mode)
    s2 = oracle.two_field_system(xyz, tets, reg, 3e-3, 0.0, 1e-5, kappa_mode=mode)
    a = oracle.solve_duplicated(sd, seq, q, (0, 1, 0), 200.0)
    b = oracle.solve_two_field(s2, seq, q, (0, 1, 0), 200.0)
    assert abs(a.normalized - b.normalized) < 1e-13 * abs(a.normalized)
    assert np.allclose(a.compartment_signals, b.compartment_signals, rtol=1e-12)
    # the literal form has dead rows exactly where no compartment cell touches
    assert s2["dead"].sum() == 4 * len(xyz) - 2 * sd["n"]


def test_layered_regions_literal_equals_duplicated():
    xyz, tets = oracle.box_mesh((-12,) * 3, (12,) * 3, 6)
    reg = oracle.region_from_centroids(xyz, tets, [lambda c: (c ** 2).sum(1) < 16,
                                                   lambda c: (c ** 2).sum(1) < 49,
                                                   lambda c: (c ** 2).sum(1) < 100])
    reg = np.where(reg == 0, 3, reg - 1).astype(np.int32)
    kp = np.zeros((4, 4))
    kp[0, 1] = kp[1, 0] = 1e-5
    kp[1, 2] = kp[2, 1] = 3e-5
    kp[2, 3] = kp[3, 2] = 5e-5
    D = np.array([1e-3, 2e-3, 3e-3, 3e-3])
    iT2 = 1.0 / np.array([5e4, 8e4, 1e5, np.inf])
    seq = oracle.PGSE(10600, 43100)
    q = oracle.bvalue_to_q(2000, seq.int4gb())
    a = oracle.solve_duplicated(oracle.duplicated_system(xyz, tets, reg, D, iT2, kp), seq, q, (1, 1, 1), 200.0)
    b = oracle.solve_two_field(oracle.two_field_system(xyz, tets, reg, D, iT2, kp), seq, q, (1, 1, 1), 200.0)
    assert abs(a.normalized - b.normalized) < 1e-13


def test_kappa_zero_decouples():
    xyz, tets = oracle.box_mesh((-5,) * 3, (5,) * 3, 5)
    reg = oracle.region_from_centroids(xyz, tets, [lambda c: c[:, 0] < 0.1])
    sd = oracle.duplicated_system(xyz, tets, reg, 3e-3, 0.0, 0.0)
    assert sd["R"].nnz == 0 or abs(sd["R"]).max() == 0.0
    # compartment blocks do not couple: no entry between dofs of different compartments
    M = (sd["M"] + sd["K"]).tocoo()
    assert np.all(sd["field"][M.row] == sd["field"][M.col])


def test_int4gb_against_sympy():
    sp = pytest.importorskip("sympy")
    s, u = sp.Symbol("s"), sp.Symbol("u")
    d, D = 10600.0, 43100.0
    T = d + D
    fs = sp.Piecewise((1., s < d), (0., s < D), (-1., s < T), (0., True))    # GCloudDmriSolver.py:188-193
    ifs = sp.integrate(fs.subs(s, u), (u, 0, s))
    ref = float(sp.integrate(ifs * ifs, (s, 0, T)))
    assert abs(oracle.PGSE(d, D).int4gb() / ref - 1) < 1e-14
    om = 2.0 * math.pi / d
    tau = T / 2.0
    fs = sp.Piecewise((0., s < 0), (sp.cos(om * s), s <= d), (0., s <= tau), (-sp.cos(om * (s - tau)), s <= d + tau),
                      (0., True))
    ifs = sp.integrate(fs.subs(s, u), (u, 0, s))
    ref = float(sp.integrate(ifs * ifs, (s, 0, T)))
    assert abs(oracle.CosOGSE(d, D).int4gb() / ref - 1) < 1e-12


def test_schedule_semantics():
    tn, to = oracle.reference_schedule(53700.0, 200.0)
    assert len(tn) == 270 and tn[0] == 0.0 and to[0] == 0.0 and np.all(to[1:] == tn[:-1])
    seq = oracle.PGSE(10600, 43100)
    assert seq.f(10599.9) == 1.0 and seq.f(10600.0) == 0.0 and seq.f(43100.0) == -1.0 and seq.f(53700.0) == 0.0
    og = oracle.CosOGSE(10600, 43100)
    assert og.f(10600.0) == pytest.approx(1.0) and og.f(0.0) == 1.0
