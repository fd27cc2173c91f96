"""Strong pseudo-periodic form -- TEST INFRASTRUCTURE ONLY.

Restates the reference's path for ``mydomain.IsDomainPeriodic = True`` with a
non-zero ``mydomain.PeriodicDir``:

* the constrained function space (``MyFunctionSpaces``, ``DmriFemLib.py:453-486``,
  ``constrained_domain=PeriodicBD``): DOLFIN pairs every vertex of an exterior
  facet that is not ``inside`` the target boundary with the vertex at
  ``map(x)`` when ``map(x)`` is ``inside`` (``PeriodicBD.inside`` / ``map``,
  ``DmriFemLib.py:325-378``; tolerance ``1e-2 * hmin``).  ``inside`` takes the
  whole min face of each periodic direction, so a max-face vertex is folded
  onto its image along the FIRST periodic direction whose max face it lies on
  (x, then y, then z) and nothing is chained: corner columns of a box end as
  three dofs, not one;
* the forms ``ThetaMethodF_sBC1c/2c`` and ``ThetaMethodL_sBC1c/2c``
  (``DmriFemLib.py:148-238``): volume integrand ``FuncF_sBC`` (first-order
  ``ift*q*(g.D grad u + grad u.D g)`` coupling of the real and imaginary parts,
  ``(g.Dg) q^2 ift^2`` and 1/T2 mass terms, diffusion), ``outer_interface`` on
  every exterior facet (``ds``, not weighted by the phase, ``+1e-16`` kept) and
  ``inner_interface`` on compartment interfaces (``|jump(phase)| dS``, normal
  ``fn0`` = outward normal of the phase-0 side, ``avg(D)`` on both sides, the
  argument ``D`` passed for both ``D0`` and ``D1``);
* the loop of ``MRI_simulation.solve`` (``DmriFemLib.py:878-915``): ``ift`` is
  ``itime_profile(t)`` in F and ``itime_profile(tp)`` in L, and L carries
  ``+theta`` (not ``1-theta``) on the explicit operator, equal at theta = 1/2.

In complex form, per compartment c with outward normal n_c on its boundary::

    A(F) = M/k + theta * (K + T + R + q^2 F^2 M_D + i q F E),
    E    = C - B,   C_ij = int (g.D grad phi_j + grad phi_j.D g) phi_i,
    B_ij = int_boundary (Dbar g . n_c) phi_i phi_j     (Dbar = avg(D) on interfaces)
    b    = (M/k - theta * (K + T + R + q^2 Fp^2 M_D + i q Fp E)) u_n

``duplicated_strong`` assembles this on one complex dof per (vertex class,
compartment) pair; ``literal_strong`` assembles the reference's real mixed
space with the phase weighting and ``ident_zeros``.  The two agree when the
compartments are periodic (a folded vertex touches the same compartments as
its master) and the literal form's phase-blind outer term, summed over the
folded space, does not reach live rows of the other compartment (it cancels
between matching periodic faces and vanishes where ``(D g).n = 0``; it does
not cancel next to the edge columns the reference's map leaves unpaired);
``duplicated_strong`` raises in the other cases, as the engine does.
``tests/test_oracle_strong.py`` checks that and pins the homogeneous box
against the closed-form product of the uniform solution.

Parity of this oracle is pinned by the literal/duplicated identity and by that
closed form: the reference ships no printed output of a strongly periodic run.
"""

import numpy as np
import scipy.sparse as sps
import scipy.sparse.linalg as spla

from .forms import (_LOCAL_FACES, _cell_tensor, _coo, element_geometry, interface_facet_matrices,
                    local_matrices)
from .periodic import hmin_of
from .sequence import reference_schedule


def _facet_table(tets):
    """(cell, local face) of every face, sorted so equal faces are adjacent."""
    n_t = len(tets)
    faces = np.sort(tets[:, _LOCAL_FACES], axis=2).reshape(-1, 3)
    cell = np.repeat(np.arange(n_t), 4)
    lface = np.tile(np.arange(4), n_t)
    order = np.lexsort((faces[:, 2], faces[:, 1], faces[:, 0]))
    return faces[order], cell[order], lface[order]


def exterior_facets(tets):
    """(cell, local face, sorted vertices) of the faces with one cell."""
    fs, cell, lface = _facet_table(tets)
    m = len(fs)
    same_next = np.zeros(m, dtype=bool)
    same_next[:-1] = np.all(fs[1:] == fs[:-1], axis=1)
    same_prev = np.zeros(m, dtype=bool)
    same_prev[1:] = same_next[:-1]
    once = ~(same_next | same_prev)
    return cell[once], lface[once], fs[once]


def outward_normal(xyz, tets, cell, lface):
    """Unit outward normal of face ``lface`` of ``cell`` (away from the opposite vertex)."""
    fv = tets[cell[:, None], _LOCAL_FACES[lface]]
    a, b, c = xyz[fv[:, 0]], xyz[fv[:, 1]], xyz[fv[:, 2]]
    n = np.cross(b - a, c - a)
    n /= np.linalg.norm(n, axis=1)[:, None]
    opp = xyz[tets[cell, lface]]
    s = np.sign(np.einsum("fk,fk->f", n, a - opp))
    return n * s[:, None]


def periodic_classes(xyz, tets, pdir, tol=None, match_tol=1e-10):
    """Master vertex of every vertex (itself when not a slave).

    DOLFIN's pairing with ``PeriodicBD`` (``DmriFemLib.py:325-378``): only
    vertices of exterior facets take part; a vertex ``inside`` the target
    boundary is a master; any other vertex x is a slave of the vertex at
    ``map(x)`` when ``map(x)`` is ``inside``.  ``map`` shifts by the box length
    along the first periodic direction whose max face holds x; the final
    ``else`` branch adds 1e7 along the non-periodic directions and never lands
    inside.  ``match_tol`` is the coordinate tolerance of the slave-master
    match (DOLFIN's ``map_tol``, 1e-10)."""
    xyz = np.asarray(xyz, dtype=np.float64)
    tets = np.asarray(tets, dtype=np.int64)
    pdir = [int(p) for p in pdir]
    if tol is None:
        tol = 1e-2 * hmin_of(xyz, tets)
    lo, hi = xyz.min(axis=0), xyz.max(axis=0)
    L = hi - lo

    def inside(p):
        return any(pdir[k] == 1 and abs(p[k] - lo[k]) < tol for k in range(3))

    _, _, fv = exterior_facets(tets)
    bverts = np.unique(fv.ravel())
    masters = [v for v in bverts if inside(xyz[v])]
    mxyz = xyz[masters] if masters else np.zeros((0, 3))
    master = np.arange(len(xyz))
    for v in bverts:
        x = xyz[v]
        if inside(x):
            continue
        y = x.copy()
        for k in range(3):
            if pdir[k] == 1 and abs(x[k] - hi[k]) < tol:
                y[k] = x[k] - L[k]
                break
        else:
            continue                                  # the else branch never lands inside
        if not inside(y):
            continue
        d = np.abs(mxyz - y).max(axis=1)
        j = int(np.argmin(d))
        if d[j] > match_tol * max(1.0, float(np.abs(y).max())):
            raise ValueError("vertex %d: no master vertex at its periodic image (mesh not periodic)" % v)
        master[v] = masters[j]
    return master


def _cell_D(D, region, n_t):
    return _cell_tensor(D, region, n_t, (3, 3))


def first_order_local(xyz, tets, region, D, g):
    """Per-cell 4x4 ``C_ij = int (g.D grad phi_j + grad phi_j.D g) phi_i`` and
    ``MD_ij = int (g.D g) phi_i phi_j`` (grad phi_j is constant and
    int phi_i = V/4)."""
    n_t = len(tets)
    vol, grads, _ = element_geometry(xyz, tets)
    Dc = _cell_D(D, region, n_t)
    gD = np.einsum("k,tkl->tl", g, Dc)                # g.D
    Dg = np.einsum("tkl,l->tk", Dc, g)                # D g
    cj = np.einsum("tl,tjl->tj", gD, grads) + np.einsum("tjk,tk->tj", grads, Dg)   # (n_t,4)
    C = (vol / 4.0)[:, None, None] * np.broadcast_to(cj[:, None, :], (n_t, 4, 4))
    gDg = np.einsum("tk,k->t", Dg, g)
    MD = (gDg * vol / 20.0)[:, None, None] * (1.0 + np.eye(4))[None]
    return C, MD


def _tri_mass(xyz, verts):
    a, b, c = xyz[verts[:, 0]], xyz[verts[:, 1]], xyz[verts[:, 2]]
    area = 0.5 * np.linalg.norm(np.cross(b - a, c - a), axis=1)
    return (area / 12.0)[:, None, None] * (1.0 + np.eye(3))[None]


def boundary_terms(xyz, tets, region, field, D, g):
    """Exterior facets: (verts, coefficient (D g).n of the owning cell, 3x3 mass)
    and interface facets: (verts, cell of the phase-0 side, cell of the other
    side, d = (avg(D) g).n0, 3x3 mass)."""
    n_t = len(tets)
    Dc = _cell_D(D, region, n_t)
    ec, el, ev = exterior_facets(tets)
    en = outward_normal(xyz, tets, ec, el)
    ecoef = np.einsum("fk,fk->f", np.einsum("fkl,l->fk", Dc[ec], g), en)
    fs, cell, lface = _facet_table(tets)
    same = np.all(fs[1:] == fs[:-1], axis=1)
    i = np.nonzero(same)[0]
    ca, cb, la, lb, iv = cell[i], cell[i + 1], lface[i], lface[i + 1], fs[i]
    m = field[ca] != field[cb]
    ca, cb, la, lb, iv = ca[m], cb[m], la[m], lb[m], iv[m]
    swap = field[ca] != 0                              # side 0 = the phase-0 cell
    c0 = np.where(swap, cb, ca)
    l0 = np.where(swap, lb, la)
    c1 = np.where(swap, ca, cb)
    n0 = outward_normal(xyz, tets, c0, l0)
    Dbar = 0.5 * (Dc[c0] + Dc[c1])
    icoef = np.einsum("fk,fk->f", np.einsum("fkl,l->fk", Dbar, g), n0)
    return (ev, ecoef, _tri_mass(xyz, ev)), (iv, c0, c1, icoef, _tri_mass(xyz, iv))


def _fold_matrix(master, n_v):
    """P (n_v x n_class) with P[v, class(v)] = 1; classes numbered by master."""
    roots = np.unique(master)
    cls = np.searchsorted(roots, master)
    P = sps.csr_matrix((np.ones(n_v), (np.arange(n_v), cls)), shape=(n_v, len(roots)))
    return P, cls, roots


def duplicated_strong(xyz, tets, region, D, invT2, kappa_pair, pdir, g, field=None, kappa_mode="facet"):
    """Complex system on one dof per live (vertex class, compartment) pair.

    Returns M, S = K + T + R, MD, E (scipy CSR, complex-ready reals), the
    signal weights ``w``, compartment of each dof and the class map."""
    xyz = np.asarray(xyz, dtype=np.float64)
    tets = np.asarray(tets, dtype=np.int64)
    region = np.asarray(region, dtype=np.int64)
    g = np.asarray(g, dtype=np.float64)
    g = g / np.linalg.norm(g)
    if field is None:
        field = region % 2
    field = np.asarray(field, dtype=np.int64)
    n_v, n_t = len(xyz), len(tets)
    master = periodic_classes(xyz, tets, pdir)
    _, cls, roots = _fold_matrix(master, n_v)
    nc = len(roots)
    nf = int(field.max()) + 1
    touch = np.zeros((n_v, nf), dtype=bool)
    touch[tets, field[:, None]] = True
    slaves = np.nonzero(master != np.arange(n_v))[0]
    bad = slaves[np.any(touch[slaves] != touch[master[slaves]], axis=1)]
    if len(bad):
        raise ValueError("compartments are not periodic: vertex %d and its master %d touch different "
                         "compartments" % (bad[0], master[bad[0]]))
    live = np.zeros((nc, nf), dtype=bool)
    live[cls[tets], field[:, None]] = True
    dof = np.full((nc, nf), -1, dtype=np.int64)
    dof[live] = np.arange(int(live.sum()))
    n = int(live.sum())
    vol, Mloc, Kloc, Tloc, _ = local_matrices(xyz, tets, region, D, invT2)
    C, MD = first_order_local(xyz, tets, region, D, g)
    cd = dof[cls[tets], field[:, None]]
    R_ = np.broadcast_to(cd[:, :, None], (n_t, 4, 4))
    C_ = np.broadcast_to(cd[:, None, :], (n_t, 4, 4))
    M = _coo(R_, C_, Mloc, n)
    S = _coo(R_, C_, Kloc + Tloc, n)
    MDm = _coo(R_, C_, MD, n)
    E = _coo(R_, C_, C, n)
    # interface permeability (same facets, kappa as in the standard form)
    ca, cb, verts, Bk = interface_facet_matrices(xyz, tets, region, field, kappa_pair, kappa_mode)
    da = dof[cls[verts], field[ca][:, None]]
    db = dof[cls[verts], field[cb][:, None]]
    rows = np.concatenate([np.repeat(da, 3, axis=1), np.repeat(db, 3, axis=1),
                           np.repeat(da, 3, axis=1), np.repeat(db, 3, axis=1)], axis=0)
    cols = np.concatenate([np.tile(da, 3), np.tile(db, 3), np.tile(db, 3), np.tile(da, 3)], axis=0)
    Bf = Bk.reshape(len(Bk), 9)
    S = S + _coo(rows, cols, np.concatenate([Bf, Bf, -Bf, -Bf], axis=0), n)
    # boundary terms of E: exterior facets of each live compartment's cells (the
    # owning cell's field), interface facets on both sides with n_c = +-n0
    (ev, ecoef, emass), (iv, c0, c1, icoef, imass) = boundary_terms(xyz, tets, region, field, D, g)
    ec, _, _ = exterior_facets(tets)
    de = dof[cls[ev], field[ec][:, None]]
    E = E - _coo(np.repeat(de, 3, axis=1), np.tile(de, 3), (ecoef[:, None, None] * emass).reshape(-1, 9), n)
    d0 = dof[cls[iv], field[c0][:, None]]
    d1 = dof[cls[iv], field[c1][:, None]]
    vals = (icoef[:, None, None] * imass).reshape(-1, 9)
    E = E - _coo(np.repeat(d0, 3, axis=1), np.tile(d0, 3), vals, n) \
          + _coo(np.repeat(d1, 3, axis=1), np.tile(d1, 3), vals, n)
    # the reference's outer term is phase-blind: on an exterior facet of a c-cell it
    # also acts on the other compartment's rows at the facet's interface vertices.
    # Summed over the folded space it must vanish (it does between matching periodic
    # faces) for a per-compartment system to equal the reference; the engine refuses
    # a gradient along which it does not (the same rule here)
    excess = {}
    dscale = np.max(np.abs(ecoef)) * np.max(emass) if len(ecoef) else 0.0
    for f in range(len(ec)):
        cf = field[ec[f]]
        for i in range(3):
            vi = ev[f, i]
            for oc in range(nf):
                if oc == cf or not touch[vi, oc]:
                    continue
                for j in range(3):
                    key = (cls[vi], oc, cls[ev[f, j]])
                    excess[key] = excess.get(key, 0.0) + ecoef[f] * emass[f, i, j]
    if any(abs(v) > 1e-10 * dscale for v in excess.values()):
        raise ValueError("(D g).n does not vanish where the phase-blind outer term reaches live rows "
                         "(the reference's literal form differs from any per-compartment system there)")
    w = np.zeros(n)
    np.add.at(w, cd.ravel(), np.repeat(vol / 4.0, 4))
    dof_class, dof_field = np.nonzero(live)
    return {"M": M.tocsr(), "S": S.tocsr(), "MD": MDm.tocsr(), "E": E.tocsr(), "w": w, "n": n,
            "field": dof_field, "class": dof_class, "class_of_vertex": cls, "master": master, "dof": dof,
            "n_fields": nf, "vertex_weight": np.bincount(tets.ravel(), weights=np.repeat(vol / 4.0, 4),
                                                         minlength=n_v)}


def _F_schedule(seq, k, loop):
    tn, to = reference_schedule(seq.T, k, loop)
    return np.array([seq.F(t) for t in tn]), np.array([seq.F(t) for t in to])


def solve_strong(sysd, seq, q, k, theta=0.5, loop="solve", u0=None, max_steps=None):
    """Crank-Nicolson loop on ``duplicated_strong`` (SuperLU per step: A depends
    on ift(t), which changes every step)."""
    M, S, MD, E = sysd["M"], sysd["S"], sysd["MD"], sysd["E"]
    Fn, Fo = _F_schedule(seq, k, loop)
    if max_steps is not None:
        Fn, Fo = Fn[:max_steps], Fo[:max_steps]
    n_v = len(sysd["vertex_weight"])
    ic = np.ones(n_v) if u0 is None else np.asarray(u0, dtype=np.float64)
    # a class takes its master's value (the constrained space interpolates the master)
    vals = ic[sysd["master"]]
    first = np.full(sysd["class"].max() + 1, -1)
    first[sysd["class_of_vertex"]] = np.arange(n_v)
    u = vals[first[sysd["class"]]].astype(np.complex128)
    S0 = float(np.dot(sysd["vertex_weight"], ic))
    Mk = (M / k).astype(np.complex128)
    Sc, MDc, Ec = S.astype(np.complex128), MD.astype(np.complex128), E.astype(np.complex128)
    for fn_, fo_ in zip(Fn, Fo):
        rhs = Mk @ u - theta * (Sc @ u + (q * fo_) ** 2 * (MDc @ u) + 1j * q * fo_ * (Ec @ u))
        A = Mk + theta * (Sc + (q * fn_) ** 2 * MDc + 1j * q * fn_ * Ec)
        u = spla.splu(A.tocsc()).solve(rhs)
    w = sysd["w"]
    sig = float(np.dot(w, u.real))
    comp = [float(np.dot(w[sysd["field"] == f], u.real[sysd["field"] == f])) for f in range(sysd["n_fields"])]
    return {"signal": sig, "S0": S0, "normalized": sig / S0, "compartments": comp, "u": u, "steps": len(Fn)}


def literal_strong(xyz, tets, region, D, invT2, kappa_pair, pdir, g, multiple=True, kappa_mode="facet"):
    """The reference's real mixed space, folded by the periodic constraint.

    Components (u0r, u0i[, u1r, u1i]) on every vertex class; global index
    comp * n_class + class.  Returns the time-independent blocks and the
    ift-dependent blocks of F (per unit q*ift and (q*ift)^2) and the 1e-16
    outer term."""
    xyz = np.asarray(xyz, dtype=np.float64)
    tets = np.asarray(tets, dtype=np.int64)
    region = np.asarray(region, dtype=np.int64)
    g = np.asarray(g, dtype=np.float64)
    g = g / np.linalg.norm(g)
    n_v, n_t = len(xyz), len(tets)
    phase = (region % 2) if multiple else np.zeros(n_t, dtype=np.int64)
    nf = 2 if multiple else 1
    master = periodic_classes(xyz, tets, pdir)
    P, cls, roots = _fold_matrix(master, n_v)
    nc = len(roots)
    N = 2 * nf * nc
    vol, Mloc, Kloc, Tloc, _ = local_matrices(xyz, tets, region, D, invT2)
    C, MD = first_order_local(xyz, tets, region, D, g)
    ct = cls[tets]
    rr = np.broadcast_to(ct[:, :, None], (n_t, 4, 4))
    cc = np.broadcast_to(ct[:, None, :], (n_t, 4, 4))

    def block(loc, chi, crow, ccol):
        return _coo(rr + crow * nc, cc + ccol * nc, loc * chi[:, None, None], N)

    Z = sps.csr_matrix((N, N))
    Mz, S, Q1, Q2 = Z, Z, Z, Z        # Q1: per unit q*ift, Q2: per unit (q*ift)^2
    for f in range(nf):
        chi = (phase == f).astype(np.float64)
        r, i = 2 * f, 2 * f + 1
        Mz = Mz + block(Mloc, chi, r, r) + block(Mloc, chi, i, i)
        # -FuncF_sBC: +K + T + (g.Dg) q^2 ift^2 on (r,r),(i,i); -q ift C on (r,i); +q ift C on (i,r)
        S = S + block(Kloc + Tloc, chi, r, r) + block(Kloc + Tloc, chi, i, i)
        Q2 = Q2 + block(MD, chi, r, r) + block(MD, chi, i, i)
        Q1 = Q1 - block(C, chi, r, i) + block(C, chi, i, r)
    # outer_interface on every exterior facet, every field (ds, no phase weight):
    # (ift q + 1e-16) (D g.n) (ui vr - ur vi)
    (ev, ecoef, emass), (iv, c0, c1, icoef, imass) = boundary_terms(xyz, tets, region, phase, D, g)
    evc = cls[ev]
    er, ecl = np.repeat(evc, 3, axis=1), np.tile(evc, 3)
    ev9 = (ecoef[:, None, None] * emass).reshape(-1, 9)
    Qeps = Z
    for f in range(nf):
        r, i = 2 * f, 2 * f + 1
        O = _coo(er + r * nc, ecl + i * nc, ev9, N) - _coo(er + i * nc, ecl + r * nc, ev9, N)
        Q1 = Q1 + O
        Qeps = Qeps + O
    if multiple:
        # kappa [u][v] on the real and imaginary parts
        ca, cb, verts, Bk = interface_facet_matrices(xyz, tets, region, phase, kappa_pair, kappa_mode)
        vc = cls[verts]
        vr_, vc_ = np.repeat(vc, 3, axis=1), np.tile(vc, 3)
        Bf = Bk.reshape(len(Bk), 9)
        for comp in (0, 1):
            a, b = comp, 2 + comp
            S = S + _coo(vr_ + a * nc, vc_ + a * nc, Bf, N) + _coo(vr_ + b * nc, vc_ + b * nc, Bf, N) \
                - _coo(vr_ + a * nc, vc_ + b * nc, Bf, N) - _coo(vr_ + b * nc, vc_ + a * nc, Bf, N)
        # first-order part of inner_interface (per unit q*ift), rows by test component:
        #   v0r: + d0 u0i            v1r: - d1 u1i
        #   v0i: - d0 u0r - (d0' - d1)/2 u1r      v1i: + (d0' + d1)/2 u1r
        # with d0 = d0' = d1 = (avg(D) g).fn0 (D passed for D0 and D1)
        d0 = d0p = d1 = icoef
        ivc = cls[iv]
        ir, icl = np.repeat(ivc, 3, axis=1), np.tile(ivc, 3)

        def fb(coef, rc, ccomp):
            return _coo(ir + rc * nc, icl + ccomp * nc, (coef[:, None, None] * imass).reshape(-1, 9), N)
        u0r, u0i, u1r, u1i = 0, 1, 2, 3
        Q1 = Q1 + fb(d0, u0r, u0i) - fb(d1, u1r, u1i) - fb(d0, u0i, u0r) - fb(0.5 * (d0p - d1), u0i, u1r) \
            + fb(0.5 * (d0p + d1), u1i, u1r)
    # ident_zeros on the folded mass (DmriFemLib.py:246,253)
    diag = np.asarray(abs(Mz).sum(axis=1)).ravel()
    dead = diag == 0.0
    Mid = Mz + sps.diags(dead.astype(np.float64))
    w_comp = []
    for f in range(nf):
        chi = (phase == f).astype(np.float64)
        w_comp.append(P.T @ np.bincount(tets.ravel(), weights=np.repeat(chi * vol / 4.0, 4), minlength=n_v))
    return {"Mid": Mid.tocsr(), "Mz": Mz.tocsr(), "S": S.tocsr(), "Q1": Q1.tocsr(), "Q2": Q2.tocsr(),
            "Qeps": Qeps.tocsr(), "nc": nc, "nf": nf, "N": N, "dead": dead, "w_comp": w_comp, "master": master,
            "class_of_vertex": cls, "P": P,
            "vertex_weight": np.bincount(tets.ravel(), weights=np.repeat(vol / 4.0, 4), minlength=n_v)}


def solve_literal_strong(sysl, seq, q, k, theta=0.5, loop="solve", u0=None, max_steps=None):
    """The reference loop on ``literal_strong``: A = Mid/k + assemble(F(ift(t))),
    b = assemble(L(u_n, ift(tp))) (``DmriFemLib.py:901-907``)."""
    Fn, Fo = _F_schedule(seq, k, loop)
    if max_steps is not None:
        Fn, Fo = Fn[:max_steps], Fo[:max_steps]
    nc, nf = sysl["nc"], sysl["nf"]
    n_v = len(sysl["vertex_weight"])
    ic = np.ones(n_v) if u0 is None else np.asarray(u0, dtype=np.float64)
    # Dirac_Delta is interpolated on the constrained space: a class holds its master's value
    cls = sysl["class_of_vertex"]
    cval = np.zeros(nc)
    cval[cls] = ic[sysl["master"]]
    u = np.zeros(sysl["N"])
    for f in range(nf):
        u[(2 * f) * nc:(2 * f + 1) * nc] = cval
    S0 = float(np.dot(sysl["vertex_weight"], ic))
    Mid, Mz, S, Q1, Q2, Qe = sysl["Mid"], sysl["Mz"], sysl["S"], sysl["Q1"], sysl["Q2"], sysl["Qeps"]
    eps = 1e-16
    for fn_, fo_ in zip(Fn, Fo):
        A = Mid / k + theta * (S + (q * fn_) ** 2 * Q2 + q * fn_ * Q1 + eps * Qe)
        b = Mz @ u / k - theta * (S @ u + (q * fo_) ** 2 * (Q2 @ u) + q * fo_ * (Q1 @ u) + eps * (Qe @ u))
        u = spla.splu(A.tocsc()).solve(b)
    comp = [float(np.dot(sysl["w_comp"][f], u[(2 * f) * nc:(2 * f + 1) * nc])) for f in range(nf)]
    sig = float(sum(comp))
    return {"signal": sig, "S0": S0, "normalized": sig / S0, "compartments": comp, "u": u, "steps": len(Fn)}


def uniform_box_signal(volume, D, invT2, seq, q, k, theta=0.5, loop="solve"):
    """Closed form of the strongly periodic homogeneous box from u0 = 1: the
    solution stays uniform (grad u = 0, C 1 = 0, the boundary terms of opposite
    faces cancel), so each step multiplies it by
    (1/k - theta (1/T2 + q^2 Fp^2 D)) / (1/k + theta (1/T2 + q^2 F^2 D))."""
    Fn, Fo = _F_schedule(seq, k, loop)
    u = 1.0
    for fn_, fo_ in zip(Fn, Fo):
        u *= (1.0 / k - theta * (invT2 + (q * fo_) ** 2 * D)) / (1.0 / k + theta * (invT2 + (q * fn_) ** 2 * D))
    return volume * u
