"""Finite-element matrices of the Bloch-Torrey weak forms -- TEST INFRASTRUCTURE ONLY.

Two restatements of the reference's forms on P1 tetrahedra:

``two_field_system`` -- literal: the real mixed space of ``MyFunctionSpaces``
(``DmriFemLib.py:453-486``), components (u0r, u0i[, u1r, u1i]) on every
vertex, cells weighted by the DG0 ``phase`` as in ``ThetaMethodF_wBC1c/2c`` and
``ThetaMethodL_wBC1c/2c`` (``DmriFemLib.py:58-145``), volume integrand
``FuncF_wBC`` (``DmriFemLib.py:41-45``), interface integrand ``icondition_wBC``
(``DmriFemLib.py:47-50``) on interior facets with ``|jump(phase)| = 1``, and the
mass matrix with ``ident_zeros`` (``DmriFemLib.py:240-254``).

``duplicated_system`` -- the same operator written as one complex unknown per
live (vertex, compartment) pair: a vertex gets a dof in compartment f when it
touches a cell of compartment f (exactly the rows that ``ident_zeros`` leaves
alone).  Interface vertices therefore appear once per side.  This is the
system the CUDA engine assembles.

Every integrand is a polynomial of degree <= 3 on each cell (``GdotX`` is
declared degree 3, ``DmriFemLib.py:33-39``), so FFC's quadrature is exact and the
closed-form P1 integrals below agree with DOLFIN up to rounding:

* mass            int phi_i phi_j          = V/20 (1 + delta_ij)
* stiffness       int D grad phi_i . grad phi_j = V grad_i^T D grad_j
* coordinate mass int x_k phi_i phi_j      = V/60 (2 x_i + S) (i = j),
                                            V/120 (x_i + x_j + S) (i != j),
  S = sum of the 4 vertex coordinates (exact: int l_i^3 = V/20,
  int l_i^2 l_j = V/60, int l_i l_j l_k = V/120)
* facet mass      int_F phi_i phi_j       = A/12 (1 + delta_ij)

Interface permeability ``kappa``: ``kappa_mode='facet'`` uses one value per
facet, taken from the region pair of its two cells (the engine's form);
``kappa_mode='cr'`` reproduces the Crouzeix-Raviart field of
``MultilayeredDiskVariablePermeability.ipynb:480-502`` (facet dof = the pair
value on interface facets, 0 elsewhere; ``avg(kappa)`` integrated exactly).
"""

import numpy as np
import scipy.sparse as sps

_LOCAL_FACES = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])  # face opposite vertex a


def element_geometry(xyz, tets):
    """Volumes (n_t,), barycentric gradients (n_t,4,3), vertex coords (n_t,4,3)."""
    X = xyz[tets]
    E = X[:, 1:, :] - X[:, :1, :]
    det = np.linalg.det(E)
    vol = np.abs(det) / 6.0
    Einv = np.linalg.inv(E)                       # grad l_k (k=1..3) = Einv[:, :, k-1]
    g = np.transpose(Einv, (0, 2, 1))             # (n_t,3,3): row k = grad l_{k+1}
    grads = np.concatenate([-g.sum(axis=1, keepdims=True), g], axis=1)
    return vol, grads, X


def _cell_tensor(values, region, n_t, shape):
    """Expand per-region scalars / per-cell arrays to per-cell arrays."""
    values = np.asarray(values, dtype=np.float64)
    if values.ndim == 0:
        return np.broadcast_to(values, (n_t,) + shape).copy() if shape == () else values * np.broadcast_to(np.eye(3), (n_t, 3, 3))
    if values.shape[0] == n_t and values.shape[1:] == shape:
        return values
    per_region = values[region]
    if shape == (3, 3) and per_region.ndim == 1:
        return per_region[:, None, None] * np.eye(3)[None]
    return per_region


def local_matrices(xyz, tets, region, D, invT2):
    """Per-cell 4x4 mass, stiffness, T2-mass and coordinate masses."""
    n_t = len(tets)
    vol, grads, X = element_geometry(xyz, tets)
    Dc = _cell_tensor(D, region, n_t, (3, 3))
    iT2 = _cell_tensor(invT2, region, n_t, ())
    eye = np.eye(4)
    Mloc = vol[:, None, None] / 20.0 * (1.0 + eye)[None]
    Kloc = vol[:, None, None] * np.einsum("tia,tab,tjb->tij", grads, Dc, grads)
    Tloc = iT2[:, None, None] * Mloc
    J = []
    for k in range(3):
        xk = X[:, :, k]
        S = xk.sum(axis=1)
        off = vol[:, None, None] / 120.0 * (xk[:, :, None] + xk[:, None, :] + S[:, None, None])
        dia = vol[:, None] / 60.0 * (2.0 * xk + S[:, None])
        Jk = off.copy()
        idx = np.arange(4)
        Jk[:, idx, idx] = dia
        J.append(Jk)
    return vol, Mloc, Kloc, Tloc, J


def interface_facets(tets, field):
    """Interior facets whose two cells lie in different compartments.

    Returns (cell_a, cell_b, local_face_a, local_face_b, verts[nf,3]).
    """
    n_t = len(tets)
    faces = np.sort(tets[:, _LOCAL_FACES], axis=2).reshape(-1, 3)
    cell = np.repeat(np.arange(n_t), 4)
    lface = np.tile(np.arange(4), n_t)
    order = np.lexsort((faces[:, 2], faces[:, 1], faces[:, 0]))
    fs = faces[order]
    same = np.all(fs[1:] == fs[:-1], axis=1)
    i = np.nonzero(same)[0]
    ca, cb = cell[order][i], cell[order][i + 1]
    la, lb = lface[order][i], lface[order][i + 1]
    verts = fs[i]
    m = field[ca] != field[cb]
    return ca[m], cb[m], la[m], lb[m], verts[m]


def all_interior_facets(tets):
    n_t = len(tets)
    faces = np.sort(tets[:, _LOCAL_FACES], axis=2).reshape(-1, 3)
    cell = np.repeat(np.arange(n_t), 4)
    lface = np.tile(np.arange(4), n_t)
    order = np.lexsort((faces[:, 2], faces[:, 1], faces[:, 0]))
    fs = faces[order]
    same = np.all(fs[1:] == fs[:-1], axis=1)
    i = np.nonzero(same)[0]
    return cell[order][i], cell[order][i + 1], lface[order][i], lface[order][i + 1], fs[i]


def _facet_area(xyz, verts):
    a, b, c = xyz[verts[:, 0]], xyz[verts[:, 1]], xyz[verts[:, 2]]
    return 0.5 * np.linalg.norm(np.cross(b - a, c - a), axis=1)


def interface_facet_matrices(xyz, tets, region, field, kappa_pair, kappa_mode="facet"):
    """Per interface facet: (cell_a, cell_b, verts[3], B[3,3]) with
    B_ij = int_F kappa phi_i phi_j."""
    ca, cb, la, lb, verts = interface_facets(tets, field)
    area = _facet_area(xyz, verts)
    kp = np.asarray(kappa_pair, dtype=np.float64)
    if kp.ndim == 0:
        kp = np.full((int(region.max()) + 1,) * 2, float(kp))
    eye3 = np.eye(3)
    if kappa_mode == "facet":
        kap = kp[region[ca], region[cb]]
        B = (kap * area / 12.0)[:, None, None] * (1.0 + eye3)[None]
        return ca, cb, verts, B
    if kappa_mode != "cr":
        raise ValueError("kappa_mode must be 'facet' or 'cr'")
    # CR field: facet dof = pair value on region-interface facets, 0 elsewhere
    # (MultilayeredDiskVariablePermeability.ipynb:480-502).
    n_t = len(tets)
    fa, fb, fla, flb, _ = all_interior_facets(tets)
    fval = np.where(region[fa] != region[fb], kp[region[fa], region[fb]], 0.0)
    cell_face_k = np.zeros((n_t, 4))
    cell_face_k[fa, fla] = fval
    cell_face_k[fb, flb] = fval

    def vertex_values(c, lf):
        # kappa_c at the 3 vertices of face lf of cell c: sum_all - 3*kappa(face opposite v)
        tot = cell_face_k[c].sum(axis=1)
        lv = _LOCAL_FACES[lf]                       # local vertex ids on the face
        opp = cell_face_k[c[:, None], lv]           # face opposite each facet vertex
        glob = tets[c[:, None], lv]
        return glob, tot[:, None] - 3.0 * opp

    ga, ka = vertex_values(ca, la)
    gb, kb = vertex_values(cb, lb)
    # reorder both to the sorted facet vertex order
    def reorder(glob, kv):
        o = np.argsort(glob, axis=1)
        return np.take_along_axis(kv, o, axis=1)
    kav = 0.5 * (reorder(ga, ka) + reorder(gb, kb))   # avg(kappa) at sorted facet verts
    # int_F l_i l_j l_l: A/10 (i=j=l), A/30 (two equal), A/60 (distinct)
    c3 = np.empty((3, 3, 3))
    for i in range(3):
        for j in range(3):
            for l in range(3):
                n_eq = len({i, j, l})
                c3[i, j, l] = {1: 1 / 10, 2: 1 / 30, 3: 1 / 60}[n_eq]
    B = area[:, None, None] * np.einsum("ijl,fl->fij", c3, kav)
    return ca, cb, verts, B


def _coo(rows, cols, vals, n):
    return sps.coo_matrix((vals.ravel(), (rows.ravel(), cols.ravel())), shape=(n, n)).tocsr()


def compartment_dofs(tets, field, n_v):
    """Live (vertex, compartment) pairs numbered vertex-major; -1 when dead."""
    nf = int(field.max()) + 1
    live = np.zeros((n_v, nf), dtype=bool)
    live[tets, field[:, None]] = True
    dof = np.full((n_v, nf), -1, dtype=np.int64)
    dof[live] = np.arange(int(live.sum()))
    return dof, nf


def duplicated_system(xyz, tets, region, D, invT2=0.0, kappa_pair=0.0, field=None,
                      kappa_mode="facet"):
    """Complex duplicated-node system.  Returns a dict with the real symmetric
    matrices M, K, T, Jx, Jy, Jz, R (scipy CSR), signal weights ``w``
    (int phi_i over the dof's compartment), ``dof`` map, compartment of each
    dof and the vertex of each dof."""
    xyz = np.asarray(xyz, dtype=np.float64)
    tets = np.asarray(tets, dtype=np.int64)
    region = np.asarray(region, dtype=np.int64)
    if field is None:
        field = region % 2                          # phase = marker % 2 (DmriFemLib.py:764)
    field = np.asarray(field, dtype=np.int64)
    n_v = len(xyz)
    dof, nf = compartment_dofs(tets, field, n_v)
    n = int((dof >= 0).sum())
    vol, Mloc, Kloc, Tloc, J = local_matrices(xyz, tets, region, D, invT2)
    cd = dof[tets, field[:, None]]                  # (n_t,4)
    R_ = np.broadcast_to(cd[:, :, None], (len(tets), 4, 4))
    C_ = np.broadcast_to(cd[:, None, :], (len(tets), 4, 4))
    out = {
        "M": _coo(R_, C_, Mloc, n), "K": _coo(R_, C_, Kloc, n), "T": _coo(R_, C_, Tloc, n),
        "Jx": _coo(R_, C_, J[0], n), "Jy": _coo(R_, C_, J[1], n), "Jz": _coo(R_, C_, J[2], n),
    }
    ca, cb, verts, B = interface_facet_matrices(xyz, tets, region, field, kappa_pair, kappa_mode)
    da = dof[verts, field[ca][:, None]]
    db = dof[verts, field[cb][:, None]]
    rows = np.concatenate([np.repeat(da, 3, axis=1), np.repeat(db, 3, axis=1),
                           np.repeat(da, 3, axis=1), np.repeat(db, 3, axis=1)], axis=0)
    cols = np.concatenate([np.tile(da, 3), np.tile(db, 3), np.tile(db, 3), np.tile(da, 3)], axis=0)
    Bf = B.reshape(len(B), 9)
    vals = np.concatenate([Bf, Bf, -Bf, -Bf], axis=0)
    out["R"] = _coo(rows, cols, vals, n)
    w = np.zeros(n)
    np.add.at(w, cd.ravel(), np.repeat(vol / 4.0, 4))
    out["w"] = w
    out["dof"] = dof
    vert_of = np.nonzero(dof >= 0)[0]
    comp_of = np.nonzero(dof >= 0)[1]
    out["vertex"] = vert_of
    out["field"] = comp_of
    out["n"] = n
    out["n_fields"] = nf
    out["volume"] = float(vol.sum())
    out["n_interface_facets"] = len(ca)
    out["vertex_weight"] = np.bincount(tets.ravel(), weights=np.repeat(vol / 4.0, 4), minlength=n_v)
    return out


def two_field_system(xyz, tets, region, D, invT2=0.0, kappa_pair=0.0, multiple=True,
                     kappa_mode="facet"):
    """Literal real mixed-space system of the reference.

    Components c = 0..2*nf-1 ordered (u0r, u0i, u1r, u1i); global index
    c*n_v + v.  Returns the pieces the time loop combines:
    ``Mid`` (mass with ident_zeros, for A), ``Mz`` (mass without, for L),
    ``S`` (K + T + R on the real/real and imag/imag blocks) and
    ``Jfuncs[k]``, the g.x coupling of ``FuncF_wBC`` per unit q*f*g_k:
    (vr,ui) = +J_k and (vi,ur) = -J_k.
    """
    xyz = np.asarray(xyz, dtype=np.float64)
    tets = np.asarray(tets, dtype=np.int64)
    region = np.asarray(region, dtype=np.int64)
    n_v = len(xyz)
    phase = (region % 2) if multiple else np.zeros(len(tets), dtype=np.int64)
    nf = 2 if multiple else 1
    ncomp = 2 * nf
    N = ncomp * n_v
    vol, Mloc, Kloc, Tloc, J = local_matrices(xyz, tets, region, D, invT2)
    T4 = tets
    rr = np.broadcast_to(T4[:, :, None], (len(tets), 4, 4))
    cc = np.broadcast_to(T4[:, None, :], (len(tets), 4, 4))

    def block(loc, chi, crow, ccol):
        return _coo(rr + crow * n_v, cc + ccol * n_v, loc * chi[:, None, None], N)

    Mz = sps.csr_matrix((N, N))
    S = sps.csr_matrix((N, N))
    Jx = [sps.csr_matrix((N, N)) for _ in range(3)]
    for f in range(nf):
        chi = (phase == f).astype(np.float64)       # (1-phase) for f=0, phase for f=1
        r, i = 2 * f, 2 * f + 1
        Mz = Mz + block(Mloc, chi, r, r) + block(Mloc, chi, i, i)
        S = S + block(Kloc + Tloc, chi, r, r) + block(Kloc + Tloc, chi, i, i)
        for k in range(3):
            # FuncF_wBC: + q f GX ui vr - q f GX ur vi  ->  as "+Jblk" in F(u,v)
            Jx[k] = Jx[k] + block(J[k], chi, r, i) - block(J[k], chi, i, r)
    if multiple:
        ca, cb, verts, B = interface_facet_matrices(xyz, tets, region, phase, kappa_pair, kappa_mode)
        vr = np.repeat(verts, 3, axis=1)
        vc = np.tile(verts, 3)
        Bf = B.reshape(len(B), 9)
        for comp in (0, 1):                          # real and imaginary parts
            a, b = comp, 2 + comp                    # u0*, u1*
            S = S + _coo(vr + a * n_v, vc + a * n_v, Bf, N) + _coo(vr + b * n_v, vc + b * n_v, Bf, N) \
                - _coo(vr + a * n_v, vc + b * n_v, Bf, N) - _coo(vr + b * n_v, vc + a * n_v, Bf, N)
    # ident_zeros on the assembled mass (DmriFemLib.py:246,253)
    diag = np.asarray(abs(Mz).sum(axis=1)).ravel()
    dead = diag == 0.0
    Mid = Mz + sps.diags(dead.astype(np.float64))
    w_comp = []
    for f in range(nf):
        chi = (phase == f).astype(np.float64)
        wv = np.bincount(tets.ravel(), weights=np.repeat(chi * vol / 4.0, 4), minlength=n_v)
        w_comp.append(wv)
    return {"Mid": Mid.tocsr(), "Mz": Mz.tocsr(), "S": S.tocsr(), "Jfuncs": [m.tocsr() for m in Jx],
            "n_v": n_v, "nf": nf, "N": N, "dead": dead, "w_comp": w_comp,
            "volume": float(vol.sum()),
            "vertex_weight": np.bincount(tets.ravel(), weights=np.repeat(vol / 4.0, 4), minlength=n_v)}
