"""Strong pseudo-periodic form in the CPU oracle (no GPU): the literal real
mixed-space restatement of the reference and the folded complex system the
engine follows agree, and the homogeneous periodic box matches its closed form."""

import math

import numpy as np
import pytest

import oracle
from oracle import strong

SEQ = oracle.PGSE(2000, 5000)


def _box_with_cylinder(n=6, half=5.0, r=2.6, per_cube=True):
    """z-cylinder through a Kuhn box.  ``per_cube``: a cube's six tetrahedra
    share the region of the cube centre, so the staircase is the same on the
    top and bottom faces (compartments periodic along z); otherwise each
    tetrahedron takes the region of its own centroid, which differs between
    the top and bottom layers."""
    xyz, tets = oracle.box_mesh((-half,) * 3, (half,) * 3, n)
    if per_cube:
        X = xyz[tets]
        c = 0.5 * (X.min(axis=1) + X.max(axis=1))
        reg = (c[:, 0] ** 2 + c[:, 1] ** 2 < r * r).astype(np.int32)
    else:
        reg = oracle.region_from_centroids(xyz, tets, [lambda c: c[:, 0] ** 2 + c[:, 1] ** 2 < r * r])
    return xyz, tets, reg


def test_periodic_classes_follow_the_reference_map():
    xyz, tets = oracle.box_mesh((0,) * 3, (4,) * 3, 4)
    m = strong.periodic_classes(xyz, tets, [1, 1, 1])
    lo, hi = 0.0, 4.0
    for v in range(len(xyz)):
        x = xyz[v]
        on_min = np.isclose(x, lo)
        if on_min.any() or not np.isclose(x, hi).any():
            assert m[v] == v                                   # masters and interior vertices
            continue
        k = int(np.nonzero(np.isclose(x, hi))[0][0])           # first max face: x, then y, then z
        y = x.copy()
        y[k] -= 4.0
        assert np.allclose(xyz[m[v]], y)
    # corner column: (xmax, ymax) folds onto (xmin, ymax), itself a master; (xmax, ymin) stays
    c = lambda p: int(np.nonzero(np.all(np.isclose(xyz, p), axis=1))[0][0])
    assert m[c([4, 4, 2])] == c([0, 4, 2])
    assert m[c([4, 0, 2])] == c([4, 0, 2]) and m[c([0, 4, 2])] == c([0, 4, 2])
    # no periodic direction: nothing folds
    assert np.array_equal(strong.periodic_classes(xyz, tets, [0, 0, 0]), np.arange(len(xyz)))
    # y only: only the ymax face folds
    my = strong.periodic_classes(xyz, tets, [0, 1, 0])
    folded = np.nonzero(my != np.arange(len(xyz)))[0]
    assert np.allclose(xyz[folded, 1], 4.0) and np.allclose(xyz[my[folded], 1], 0.0)


@pytest.mark.parametrize("pdir,g", [([1, 0, 0], (1, 0, 0)), ([0, 1, 0], (0, 1, 0)), ([0, 0, 1], (0, 0, 1))])
def test_homogeneous_box_closed_form(pdir, g):
    """One periodic direction along g: the boundary terms of the two periodic
    faces cancel in the folded space and the other faces have g.n = 0, so the
    solution from u0 = 1 stays uniform and the signal is the closed-form product."""
    xyz, tets = oracle.box_mesh((0,) * 3, (6,) * 3, 5)
    reg = np.zeros(len(tets), np.int32)
    D, iT2, k = 2e-3, 1.0 / 8e4, 100.0
    q = oracle.bvalue_to_q(3000, SEQ.int4gb())
    sd = strong.duplicated_strong(xyz, tets, reg, D, iT2, 0.0, pdir, g, field=reg)
    r = strong.solve_strong(sd, SEQ, q, k)
    exact = strong.uniform_box_signal(216.0, D, iT2, SEQ, q, k)
    assert abs(r["signal"] - exact) < 1e-11 * abs(exact)
    assert np.abs(r["u"] - r["u"][0]).max() < 1e-12 * abs(r["u"][0])
    # and it is close to the continuous free-diffusion attenuation exp(-bD - TE/T2)
    assert abs(r["normalized"] / math.exp(-3000 * D - SEQ.T * iT2) - 1.0) < 2e-2
    ll = strong.literal_strong(xyz, tets, reg, D, iT2, 0.0, pdir, g, multiple=False)
    b = strong.solve_literal_strong(ll, SEQ, q, k)
    assert abs(b["signal"] - exact) < 1e-11 * abs(exact)


def test_several_directions_keep_the_reference_edge_columns():
    """With two or three periodic directions the reference's map leaves the
    edge columns (xmax, ymin) and (xmin, ymin) unpaired (both are masters), so
    a gradient with components across those edges does not keep the box
    uniform: the signal departs from the closed form, identically in both
    restatements."""
    xyz, tets = oracle.box_mesh((0,) * 3, (6,) * 3, 5)
    reg = np.zeros(len(tets), np.int32)
    q = oracle.bvalue_to_q(3000, SEQ.int4gb())
    g = (1, 2, 0.5)
    sd = strong.duplicated_strong(xyz, tets, reg, 2e-3, 0.0, 0.0, [1, 1, 1], g, field=reg)
    r = strong.solve_strong(sd, SEQ, q, 100.0)
    exact = strong.uniform_box_signal(216.0, 2e-3, 0.0, SEQ, q, 100.0)
    assert abs(r["signal"] - exact) > 1e-3 * exact
    ll = strong.literal_strong(xyz, tets, reg, 2e-3, 0.0, 0.0, [1, 1, 1], g, multiple=False)
    b = strong.solve_literal_strong(ll, SEQ, q, 100.0)
    assert abs(b["signal"] - r["signal"]) < 1e-11 * abs(r["signal"])
    # 6^3 vertices: 5 per axis are unique after folding, plus the unpaired edge columns
    m = strong.periodic_classes(xyz, tets, [1, 1, 1])
    assert len(np.unique(m)) > 5 ** 3


@pytest.mark.parametrize("pdir,g", [([1, 1, 1], (1, 0.4, 0.3)), ([1, 1, 0], (0.6, 1, 0))])
def test_literal_equals_duplicated_two_compartments(pdir, g):
    """z-cylinder through the box: with every exterior facet periodic (or with
    (Dg).n = 0 on the non-periodic z faces) the literal form's dead rows
    decouple and both restatements give the same signal."""
    xyz, tets, reg = _box_with_cylinder()
    D = np.array([3e-3, 1.5e-3])
    iT2 = np.array([0.0, 1.0 / 6e4])
    q = oracle.bvalue_to_q(2500, SEQ.int4gb())
    sd = strong.duplicated_strong(xyz, tets, reg, D, iT2, 2e-5, pdir, g)
    sl = strong.literal_strong(xyz, tets, reg, D, iT2, 2e-5, pdir, g)
    a = strong.solve_strong(sd, SEQ, q, 100.0)
    b = strong.solve_literal_strong(sl, SEQ, q, 100.0)
    assert abs(a["normalized"] - b["normalized"]) < 1e-12
    assert np.allclose(a["compartments"], b["compartments"], rtol=1e-11, atol=1e-12)
    # every live (class, compartment) pair is a live literal row
    assert int((~sl["dead"]).sum()) == 2 * sd["n"]


def test_literal_differs_when_a_non_periodic_face_sees_the_gradient():
    """With g.n != 0 on a non-periodic face the literal form couples the dead
    rows of the other compartment there (its outer term is not phase
    weighted): no per-compartment system equals it, and the duplicated system
    refuses that gradient, as the engine does."""
    xyz, tets, reg = _box_with_cylinder()
    g = (0.3, 0.2, 1.0)
    with pytest.raises(ValueError, match="phase-blind"):
        strong.duplicated_strong(xyz, tets, reg, 3e-3, 0.0, 2e-5, [1, 1, 0], g)
    sl = strong.literal_strong(xyz, tets, reg, 3e-3, 0.0, 2e-5, [1, 1, 0], g)
    dead = np.nonzero(sl["dead"])[0]
    live = np.nonzero(~sl["dead"])[0]
    # the literal form's first-order block couples live rows to dead columns
    assert np.abs(sl["Q1"][live][:, dead]).max() > 0.0


def test_non_periodic_compartments_are_rejected():
    """Per-tetrahedron staircase: the top-face layer puts other tetrahedra in
    the cylinder than the bottom-face layer, so a folded vertex touches other
    compartments than its master.  The literal form then differs from any
    per-compartment system (its outer term is phase-blind); the duplicated
    system refuses the mesh."""
    xyz, tets, reg = _box_with_cylinder(per_cube=False)
    with pytest.raises(ValueError, match="not periodic"):
        strong.duplicated_strong(xyz, tets, reg, 3e-3, 0.0, 2e-5, [0, 0, 1], (0, 0, 1))
    strong.duplicated_strong(xyz, tets, reg, 3e-3, 0.0, 2e-5, [1, 1, 0], (1, 0, 0))   # x, y faces: one compartment


def test_operator_structure():
    """One compartment, constant D, periodic along g (g.n = 0 on the other
    faces): C + C^T equals the boundary matrix of the folded space (zero), so E
    is skew and A is Hermitian;
    with two compartments and unequal D it is neither Hermitian nor complex
    symmetric (the engine's solver is BiCGSTAB)."""
    xyz, tets = oracle.box_mesh((0,) * 3, (4,) * 3, 4)
    reg = np.zeros(len(tets), np.int32)
    sd = strong.duplicated_strong(xyz, tets, reg, 3e-3, 0.0, 0.0, [1, 0, 0], (1, 0, 0), field=reg)
    E = sd["E"].toarray()
    assert np.abs(E + E.T).max() < 1e-15 * np.abs(E).max() * 10
    xyz, tets, reg = _box_with_cylinder(n=4)
    sd = strong.duplicated_strong(xyz, tets, reg, np.array([3e-3, 1e-3]), 0.0, 1e-5, [1, 1, 1], (1, 1, 0))
    E = sd["E"].toarray()
    assert np.abs(E + E.T).max() > 1e-6 * np.abs(E).max()
    assert np.abs(E - E.T).max() > 1e-6 * np.abs(E).max()


def test_literal_equals_duplicated_with_a_tensor_field():
    """Per-cell anisotropic tensor (symmetric, varying per cube column so it is
    periodic across the z faces) and per-cell 1/T2: both restatements agree."""
    xyz, tets, reg = _box_with_cylinder(n=6)
    X = xyz[tets].min(axis=1)
    col = (np.rint((X[:, 0] + 5.0) / (10.0 / 6)) * 6 + np.rint((X[:, 1] + 5.0) / (10.0 / 6))).astype(int)
    rng = np.random.default_rng(4)
    base = np.where(reg == 1, 1.5e-3, 3e-3)
    A = rng.normal(size=(36, 3, 3)) * 0.2
    Dt = base[:, None, None] * (np.eye(3)[None] + 0.25 * (A[col] + np.transpose(A[col], (0, 2, 1))))
    iT2 = (1.0 / (5e4 + 5e4 * rng.random(36)))[col]
    q = oracle.bvalue_to_q(2000, SEQ.int4gb())
    g = (0.5, 0.7, 0.3)
    sd = strong.duplicated_strong(xyz, tets, reg, Dt, iT2, 2e-5, [1, 1, 1], g)
    sl = strong.literal_strong(xyz, tets, reg, Dt, iT2, 2e-5, [1, 1, 1], g)
    a = strong.solve_strong(sd, SEQ, q, 100.0)
    b = strong.solve_literal_strong(sl, SEQ, q, 100.0)
    assert abs(a["normalized"] - b["normalized"]) < 1e-12
    assert np.allclose(a["compartments"], b["compartments"], rtol=1e-11, atol=1e-12)


def test_phase_blind_term_reaching_live_rows_is_refused():
    """On the 5-cube box the cylinder's interface vertices on the z faces share
    exterior facets with edge vertices the reference's map leaves unpaired
    ((x, ymin, z) columns are masters), so the phase-blind outer term does not
    cancel between the z faces: the literal form differs from the per-compartment
    system along g_z, which refuses it (as the engine does); g in the x-y plane is
    exact."""
    xyz, tets, reg = _box_with_cylinder(n=5)
    q = oracle.bvalue_to_q(2000, SEQ.int4gb())
    with pytest.raises(ValueError, match="phase-blind"):
        strong.duplicated_strong(xyz, tets, reg, 3e-3, 0.0, 2e-5, [1, 1, 1], (0.5, 0.7, 0.3))
    sl = strong.literal_strong(xyz, tets, reg, 3e-3, 0.0, 2e-5, [1, 1, 1], (0.5, 0.7, 0.3))
    sd0 = strong.duplicated_strong(xyz, tets, reg, 3e-3, 0.0, 2e-5, [1, 1, 1], (0.5, 0.7, 0.0))
    sl0 = strong.literal_strong(xyz, tets, reg, 3e-3, 0.0, 2e-5, [1, 1, 1], (0.5, 0.7, 0.0))
    a = strong.solve_strong(sd0, SEQ, q, 100.0, max_steps=20)
    b = strong.solve_literal_strong(sl0, SEQ, q, 100.0, max_steps=20)
    assert abs(a["normalized"] - b["normalized"]) < 1e-12
    assert sl["N"] > 0
