"""Weak pseudo-periodic boundary term -- TEST INFRASTRUCTURE ONLY.

Restates the penalty form the reference uses when ``mydomain.PeriodicDir`` is
set and ``IsDomainPeriodic`` is False (``DmriFemLib.py``):

* implicit form: ``theta * kappa_e * (ur*vr + ui*vi) * ds``
  (``ThetaMethodF_wBC1c``, ``:79-93``; two compartments weighted by the
  cell's phase, ``ThetaMethodF_wBC2c``, ``:125-145``);
* explicit form: ``(1-theta) * kappa_e * (ubc_r*vr + ubc_i*vi) * ds``
  (``ThetaMethodL_wBC1c``, ``:58-77``; ``ThetaMethodL_wBC2c``, ``:96-122``);
* ``ubc`` is ``WeakPseudoPeriodic_1c/2c.eval`` (``:386-451``, ``:256-323``):
  on a periodic face, u_n at the mirror point on the opposite face rotated by
  ``exp(i * qvalue * (g . ln) * ift)`` with ``ln`` the shift to the mirror
  point and ``ift = itime_profile(tp)``; directions x, y, z in turn, min face
  then max face, tolerance 1e-7, a later match replacing an earlier one;
  zero elsewhere;
* ``kappa_e = kappa_e_scalar * [x within tol of a periodic face]`` with
  ``kappa_e_scalar = 3e-3 / hmin`` and ``tol = 1e-2 * hmin``
  (``WeakPseudoPeridicMarker``, ``:596-610``; ``MyDomain``, ``:587-589``).

``kappa_e`` and ``ubc`` are degree-1 expressions, so each is its P1
interpolant on a cell and the facet integrals are exact cubic integrals:
int l_a l_b l_c over a triangle = |F|/10, |F|/30 or |F|/60 for three, two or no
equal indices.  The mirror value is the P1 interpolant on the boundary
triangle of the opposite face that contains the mirror point (the one with the
largest smallest barycentric coordinate), from the dofs of the boundary
vertex's own compartment (a triangle vertex without a dof there adds zero).
"""

import numpy as np
import scipy.sparse as sps

_LOCAL_FACES = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])


def hmin_of(xyz, tets):
    """Smallest cell diameter (largest vertex distance of a cell)."""
    X = xyz[tets]
    h = np.zeros(len(tets))
    for a in range(4):
        for b in range(a + 1, 4):
            h = np.maximum(h, np.linalg.norm(X[:, a] - X[:, b], axis=1))
    return float(h.min())


def exterior_facets(tets):
    """(cell, three vertices) of the faces that belong to one cell only."""
    f = tets[:, _LOCAL_FACES]                        # (n_t, 4, 3)
    key = np.sort(f, axis=2).reshape(-1, 3)
    _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    once = cnt[inv.ravel()] == 1
    cells = np.repeat(np.arange(len(tets)), 4)[once]
    return cells, f.reshape(-1, 3)[once]


def _tri3(a, b, c):
    if a == b == c:
        return 1.0 / 10.0
    if a == b or b == c or a == c:
        return 1.0 / 30.0
    return 1.0 / 60.0


def weak_periodic(xyz, tets, field, dof, periodic_dir):
    """Boundary penalty matrix ``B`` (n x n, real) and the mirror map of every
    dof: ``mirror[j] = (dofs k, weights, shift)``.  ``dof`` is the (vertex,
    compartment) -> dof map of ``forms.compartment_dofs``."""
    xyz = np.asarray(xyz, np.float64)
    tets = np.asarray(tets, np.int64)
    field = np.asarray(field, np.int64)
    pdir = [int(bool(d)) for d in periodic_dir]
    n = int((dof >= 0).sum())
    lo, hi = xyz.min(axis=0), xyz.max(axis=0)
    hmin = hmin_of(xyz, tets)
    tol, ks = 1e-2 * hmin, 3e-3 / hmin
    on = np.zeros(len(xyz), bool)
    for d in range(3):
        if pdir[d]:
            on |= (xyz[:, d] < lo[d] + tol) | (xyz[:, d] > hi[d] - tol)
    kap = np.where(on, ks, 0.0)

    cells, fv = exterior_facets(tets)
    rows, cols, vals = [], [], []
    for c, f in zip(cells, fv):
        ka = kap[f]
        if not ka.any():
            continue
        area = 0.5 * np.linalg.norm(np.cross(xyz[f[1]] - xyz[f[0]], xyz[f[2]] - xyz[f[0]]))
        dd = dof[f, field[c]]
        for i in range(3):
            for j in range(3):
                rows.append(dd[i])
                cols.append(dd[j])
                vals.append(area * sum(ka[a] * _tri3(a, i, j) for a in range(3)))
    B = sps.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()

    # boundary triangles of each periodic face
    planes = {}
    for d in range(3):
        if not pdir[d]:
            continue
        for side, val in ((0, lo[d]), (1, hi[d])):
            sel = np.all(np.abs(xyz[fv][:, :, d] - val) <= tol, axis=1)
            planes[(d, side)] = fv[sel]

    def locate(d, side, p):
        tri = planes[(d, side)]
        au, av = (d + 1) % 3, (d + 2) % 3
        A = xyz[tri[:, 0]][:, [au, av]]
        Bv = xyz[tri[:, 1]][:, [au, av]]
        C = xyz[tri[:, 2]][:, [au, av]]
        q = p[[au, av]]
        det = (Bv[:, 0] - A[:, 0]) * (C[:, 1] - A[:, 1]) - (C[:, 0] - A[:, 0]) * (Bv[:, 1] - A[:, 1])
        l1 = ((q[0] - A[:, 0]) * (C[:, 1] - A[:, 1]) - (C[:, 0] - A[:, 0]) * (q[1] - A[:, 1])) / det
        l2 = ((Bv[:, 0] - A[:, 0]) * (q[1] - A[:, 1]) - (q[0] - A[:, 0]) * (Bv[:, 1] - A[:, 1])) / det
        lam = np.stack([1.0 - l1 - l2, l1, l2], axis=1)
        best = int(np.argmax(lam.min(axis=1)))
        w = lam[best].copy()
        w[np.abs(w) <= 1e-13] = 0.0
        return tri[best], w

    vert_of, comp_of = np.nonzero(dof >= 0)
    order = np.argsort(dof[vert_of, comp_of])
    vert_of, comp_of = vert_of[order], comp_of[order]
    mirror = {}
    cache = {}
    for j in range(n):
        v, c = vert_of[j], comp_of[j]
        x = xyz[v]
        hit = None
        for d in range(3):
            if not pdir[d]:
                continue
            if abs(x[d] - lo[d]) <= 1e-7:
                hit = (d, 1)
            if abs(x[d] - hi[d]) <= 1e-7:
                hit = (d, 0)
        if hit is None:
            continue
        d, side = hit
        if v not in cache:
            p = x.copy()
            p[d] = hi[d] if side else lo[d]
            shift = np.zeros(3)
            shift[d] = p[d] - x[d]
            tri, w = locate(d, side, p)
            cache[v] = (tri, w, shift)
        tri, w, shift = cache[v]
        ks_, ws_ = [], []
        for t, lam in zip(tri, w):
            k = dof[t, c]
            if lam != 0.0 and k >= 0:
                ks_.append(int(k))
                ws_.append(float(lam))
        mirror[j] = (np.array(ks_, np.int64), np.array(ws_), shift)
    return {"B": B, "mirror": mirror, "kappa_e": ks, "hmin": hmin}


def ubc(per, u, q, g, F):
    """Nodal values of ``ubc`` for the state ``u`` (complex per dof), q-value
    ``q``, unit gradient direction ``g`` and ``F = itime_profile(tp)``."""
    out = np.zeros(len(u), np.complex128)
    for j, (ks_, ws_, shift) in per["mirror"].items():
        out[j] = np.exp(1j * q * float(np.dot(g, shift)) * F) * np.dot(ws_, u[ks_])
    return out
