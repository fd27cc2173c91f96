"""Weak pseudo-periodic boundaries in the CPU oracle (no GPU): the free-diffusion
limit the reference quotes for a periodic direction (exp(-bD),
MultilayeredStructures.ipynb:535), b = 0 invariance, and the mirror map of a
box whose opposite faces match."""

import numpy as np

import oracle
from oracle import forms
from oracle.periodic import weak_periodic, exterior_facets

L, D = 5.0, 2e-3
SEQ = oracle.PGSE(1000.0, 10000.0)


def box(n):
    xyz, tets = oracle.box_mesh([-L, -L, -L], [L, L, L], n)
    reg = np.zeros(len(tets), np.int64)
    return xyz, tets, reg, forms.duplicated_system(xyz, tets, reg, [D])


def signal(sysd, per, b, g=(1.0, 0.0, 0.0), k=50.0):
    q = oracle.bvalue_to_q(b, SEQ.int4gb())
    return oracle.solve_duplicated(sysd, SEQ, q, g, k, periodic=per).normalized


def test_free_diffusion_limit():
    """Periodic along the gradient: the signal approaches exp(-bD) as the mesh is
    refined (weak form, first order), far closer than the restricted (Neumann) box."""
    free = np.exp(-500.0 * D)
    errs = []
    for n in (8, 12):
        xyz, tets, reg, sysd = box(n)
        per = weak_periodic(xyz, tets, reg, sysd["dof"], [1, 0, 0])
        errs.append(abs(signal(sysd, per, 500.0) - free))
        if n == 8:
            neumann = abs(signal(sysd, None, 500.0) - free)
    assert errs[1] < 0.6 * errs[0]
    assert errs[1] < 0.02 and neumann > 0.3


def test_b0_stays_one():
    """q = 0: u = 1 satisfies both the bulk and the (theta = 1/2) penalty step."""
    xyz, tets, reg, sysd = box(6)
    per = weak_periodic(xyz, tets, reg, sysd["dof"], [1, 1, 1])
    assert abs(signal(sysd, per, 0.0) - 1.0) < 1e-12


def test_mirror_map_of_matching_faces():
    """A box with matching faces: every vertex on a periodic face mirrors to the
    opposite vertex with weight 1 and a shift of one box length; kappa_e = 3e-3/hmin."""
    xyz, tets, reg, sysd = box(4)
    per = weak_periodic(xyz, tets, reg, sysd["dof"], [0, 1, 0])
    dof = sysd["dof"][:, 0]
    on_face = np.abs(np.abs(xyz[:, 1]) - L) < 1e-9
    assert len(per["mirror"]) == int(on_face.sum())
    for v in np.nonzero(on_face)[0]:
        ks, ws, shift = per["mirror"][dof[v]]
        target = xyz[v].copy()
        target[1] = -target[1]
        assert len(ks) == 1 and ws[0] == 1.0
        assert np.allclose(xyz[sysd["vertex"][ks[0]]], target)
        assert np.allclose(shift, [0.0, target[1] - xyz[v, 1], 0.0])
    assert abs(per["kappa_e"] - 3e-3 / per["hmin"]) < 1e-15
    # B lives on the exterior facets of the two y faces (kappa_e is 1 on their
    # vertices, including their edges with the other faces)
    cells, fv = exterior_facets(tets)
    assert len(fv) == 6 * 4 * 4 * 2
    assert np.allclose(per["B"].toarray(), per["B"].toarray().T)


def test_mirror_map_two_compartments():
    """Across the z faces of a box with a z-cylinder every boundary dof mirrors to
    the opposite vertex, with weight 1, in its own compartment -- or to nothing
    when that vertex has no dof in the compartment (the Kuhn split is not mirror-
    symmetric in z, so the centroid staircase of the cylinder differs slightly
    between the two faces)."""
    xyz, tets = oracle.box_mesh([-L, -L, -L], [L, L, L], 6)
    mid = xyz[tets].mean(axis=1)
    reg = (mid[:, 0] ** 2 + mid[:, 1] ** 2 < 2.5 ** 2).astype(np.int64)
    sysd = forms.duplicated_system(xyz, tets, reg, [D, D], 0.0, np.array([[0.0, 1e-5], [1e-5, 0.0]]))
    dof = sysd["dof"]
    per = weak_periodic(xyz, tets, reg % 2, dof, [0, 0, 1])
    on_face = np.abs(np.abs(xyz[:, 2]) - L) < 1e-9
    assert len(per["mirror"]) == int(sum((dof[v] >= 0).sum() for v in np.nonzero(on_face)[0]))
    where = {tuple(np.round(p, 9)): v for v, p in enumerate(xyz)}
    matched = empty = 0
    for j, (ks, ws, shift) in per["mirror"].items():
        v, c = sysd["vertex"][j], sysd["field"][j]
        target = xyz[v].copy()
        target[2] = -target[2]
        w = where[tuple(np.round(target, 9))]
        if dof[w, c] >= 0:
            assert list(ks) == [dof[w, c]] and ws[0] == 1.0
            matched += 1
        else:
            assert len(ks) == 0
            empty += 1
    assert matched > 10 * empty and sum(int((dof[v] >= 0).sum() == 2) for v in np.nonzero(on_face)[0]) > 0
