"""Reference-compatible solver API on top of libbtgpu.

Names, attributes and call order follow the reference's Python API
(van-dang/DMRI-FEM-Cloud ``DmriFemLib.py``):

    mri_simu = MRI_simulation(); mri_para = MRI_parameters()
    mri_para.bvalue = 1000; mri_para.delta, mri_para.Delta = 10600, 43100
    mri_para.set_gradient_dir(mymesh, 0, 1, 0)
    mri_para.T = mri_para.Delta + mri_para.delta
    mri_para.profile = sequences.pgse(mri_para.delta, mri_para.Delta)   # or fs_sym
    mri_para.Apply()
    mri_simu.k = 200
    mydomain = MyDomain(mymesh, mri_para)
    mydomain.phase = phase; mydomain.IsDomainMultiple = True; mydomain.kappa = 1e-5
    mydomain.PeriodicDir = [0, 0, 0]; mydomain.IsDomainPeriodic = False
    mydomain.Apply(); mydomain.D = 3e-3
    mri_simu.solve(mydomain, mri_para, linsolver)
    PostProcessing(mydomain, mri_para, mri_simu, None)

The DOLFIN ``Mesh`` is replaced by :class:`Mesh` (vertex coordinates, tets and
optional cell markers).  The linear solver argument is any object with a
``parameters`` mapping (e.g. :class:`KrylovSolver`); ``relative_tolerance`` and
``maximum_iterations`` map to the Krylov stopping rule.  Pseudo-periodic
boundaries (``PeriodicDir != [0,0,0]``) are imposed weakly when
``IsDomainPeriodic`` is False and strongly (constrained periodic function space,
FP64 BiCGSTAB; the mesh must be periodic) when it is True, as in the reference.
"""

import math
import os
import sys
import time

import numpy as np

from . import _native
from . import sequences as seqs


def _compact_markers(mk):
    """Marker values renumbered to small non-negative integers, in increasing
    order, each keeping its parity (phase = marker % 2 is preserved)."""
    mk = np.asarray(mk, np.int64)
    out = np.empty(len(mk), np.int32)
    nxt = {0: 0, 1: 1}
    for v in np.unique(mk):
        par = int(v) % 2
        out[mk == v] = nxt[par]
        nxt[par] += 2
    return out


class Mesh:
    """Tetrahedral mesh: xyz[n_v,3] (um), tets[n_t,4], optional markers[n_t]."""

    def __init__(self, xyz, tets, markers=None):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.tets = np.ascontiguousarray(tets, dtype=np.int32)
        if self.xyz.ndim != 2 or self.xyz.shape[1] != 3:
            raise ValueError("xyz must be (n_vertices, 3): only 3-D tetrahedral meshes are supported")
        if self.tets.ndim != 2 or self.tets.shape[1] != 4:
            raise ValueError("tets must be (n_cells, 4)")
        self.markers = None if markers is None else np.ascontiguousarray(markers, dtype=np.int32)

    @classmethod
    def read(cls, path, markers=None, compact_markers=False):
        """Mesh from a gmsh ``.msh`` / DOLFIN ``.xml`` file (plain or ``.zip``).

        Cell markers are the file's own (gmsh physical tags, DOLFIN domains);
        ``markers`` may instead name a DOLFIN mesh-function file (the
        ``pmk_*.xml`` of ``GetPartitionMarkers``, ``DmriFemLib.py:689``) or be an
        array.  ``compact_markers`` renumbers the marker values to 0..k-1 in
        increasing order while keeping each value's parity (so the reference's
        phase = marker % 2 is unchanged)."""
        from . import meshfiles
        name = str(path)
        stem = name[:-4] if name.endswith(".zip") else name
        if stem.endswith(".msh"):
            d = meshfiles.read_msh(path)
        elif stem.endswith(".xml"):
            d = meshfiles.read_dolfin_xml(path)
        else:
            raise ValueError("unknown mesh file type: %s (expected .msh or .xml, optionally .zip)" % name)
        mk = d["markers"]
        if isinstance(markers, (str, os.PathLike)):
            mk = meshfiles.read_mesh_function(markers, len(d["tets"]))
        elif markers is not None:
            mk = np.asarray(markers, np.int32)
        if mk is not None and compact_markers:
            mk = _compact_markers(mk)
        return cls(d["xyz"], d["tets"], mk)

    def num_vertices(self):
        return len(self.xyz)

    def num_cells(self):
        return len(self.tets)

    def coordinates(self):
        return self.xyz

    def cell_edge_lengths(self):
        X = self.xyz[self.tets]
        pairs = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
        return np.stack([np.linalg.norm(X[:, a] - X[:, b], axis=1) for a, b in pairs], axis=1)

    def hmin(self):
        """min over cells of the largest vertex distance (DOLFIN Cell::h)."""
        return float(self.cell_edge_lengths().max(axis=1).min())

    def hmax(self):
        return float(self.cell_edge_lengths().max(axis=1).max())


def project_cell_values(mymesh, cell_values, rtol=1e-14):
    """L2 projection of a per-cell (DG0) field onto P1: the vertex values x with
    M x = b, M the P1 mass matrix of the whole mesh and b_i = sum over cells c
    of v_c |c| / 4.  This is the reference's ``project(disc_ic, mydomain.V)``
    that turns a per-compartment initial condition into the continuous
    ``Dirac_Delta`` handed to ``MRI_simulation.solve``
    (``DiscontinuousInitialCondition.ipynb``, cell 10).  Host-side set-up only
    (Jacobi-CG on the consistent mass matrix, which is well conditioned).
    Returns one value per vertex, for ``solve(..., ic=...)``."""
    import scipy.sparse as sps
    import scipy.sparse.linalg as spla
    xyz, tets = mymesh.xyz, mymesh.tets.astype(np.int64)
    v = np.asarray(cell_values, np.float64).reshape(len(tets))
    E = xyz[tets[:, 1:]] - xyz[tets[:, :1]]
    vol = np.abs(np.linalg.det(E)) / 6.0
    loc = (vol / 20.0)[:, None, None] * (1.0 + np.eye(4))[None]
    rr = np.broadcast_to(tets[:, :, None], loc.shape).ravel()
    cc = np.broadcast_to(tets[:, None, :], loc.shape).ravel()
    n_v = len(xyz)
    M = sps.coo_matrix((loc.ravel(), (rr, cc)), shape=(n_v, n_v)).tocsr()
    b = np.bincount(tets.ravel(), weights=np.repeat(v * vol / 4.0, 4), minlength=n_v)
    d = M.diagonal()
    if np.any(d <= 0.0):
        raise ValueError("project_cell_values: a vertex belongs to no cell")
    P = spla.LinearOperator(M.shape, matvec=lambda x: x / d, dtype=np.float64)
    x, info = spla.cg(M, b, x0=b / (4.0 * d), rtol=rtol, atol=0.0, maxiter=1000, M=P)
    if info != 0:
        raise RuntimeError("project_cell_values: CG did not converge")
    return x


class KrylovSolver:
    """Stand-in for DOLFIN's ``KrylovSolver`` (``GCloudDmriSolver.py:219-222``).

    The method and preconditioner names are recorded; the engine always runs
    Jacobi-preconditioned COCG on the complex-symmetric CN system.
    ``parameters['precision']`` selects 'fp64' (default) or 'mixed'.
    """

    def __init__(self, method="cocg", preconditioner="jacobi"):
        self.method = method
        self.preconditioner = preconditioner
        self.parameters = {"relative_tolerance": 1e-12, "absolute_tolerance": 0.0,
                           "maximum_iterations": 2000, "precision": "fp64"}


class MRI_parameters:
    """``MRI_parameters`` (``DmriFemLib.py:800-858``)."""

    def __init__(self):
        self.bvalue = None
        self.gvalue = None
        self.qvalue = None
        self.gdir = np.array([1.0, 0.0, 0.0])
        self.nperiod = 0
        self.T2 = 1e16
        self.T = None
        self.delta = None
        self.Delta = None
        self.profile = None   # a sequences.TimeProfile
        self.fs_sym = None    # optional sympy Piecewise in the symbol self.s
        self.s = None
        try:  # the reference builds fs_sym from self.s
            import sympy as _sp
            self.s = _sp.Symbol("s")
        except ImportError:
            pass

    def set_gradient_dir(self, mymesh, g0, g1, g2):
        g = np.array([g0, g1, g2], dtype=np.float64)
        nrm = float(np.linalg.norm(g))
        if not nrm > 1e-10:
            raise ValueError("|g|=0! Please check again the gradient directions!")
        self.gdir = g / nrm

    # -- time profile -------------------------------------------------------
    def _ensure_profile(self):
        if self.profile is not None:
            return
        if self.fs_sym is not None:
            self.profile = _SympyProfile(self.fs_sym, self.s, self.T)
            return
        if self.delta is not None and self.Delta is not None:
            self.profile = seqs.pgse(self.delta, self.Delta)
            return
        raise ValueError("set mri_para.profile (or fs_sym, or delta/Delta for PGSE)")

    def time_profile(self, t):
        self._ensure_profile()
        return self.profile.f(t)

    def itime_profile(self, t):
        self._ensure_profile()
        return self.profile.F(t)

    def integral_term_for_gb(self):
        self._ensure_profile()
        self.int4gb = float(self.profile.int4gb())

    def convert_b2q(self):
        self.qvalue = seqs.b_to_q(self.bvalue, self.int4gb)
        return self.qvalue

    def convert_q2b(self):
        self.bvalue = seqs.q_to_b(self.qvalue, self.int4gb)
        return self.bvalue

    def Apply(self):
        self._ensure_profile()
        if self.T is None:
            self.T = self.profile.T
        self.integral_term_for_gb()
        if self.bvalue is not None:
            self.qvalue = self.convert_b2q()
            self.gvalue = seqs.q_to_g(self.qvalue)
        elif self.gvalue is not None:
            self.qvalue = seqs.g_to_q(self.gvalue)
            self.bvalue = self.convert_q2b()
        else:
            raise ValueError("bvalue or gvalue need to be specified.")


class _SympyProfile:
    """Wraps a sympy Piecewise exactly as the reference evaluates it
    (``time_profile`` / ``itime_profile_sym`` / ``integral_term_for_gb``)."""

    def __init__(self, fs_sym, s, T):
        import sympy as sp
        self._sp = sp
        self.fs_sym = fs_sym
        self.s = s
        self.T = float(T)
        u = sp.Symbol("u")
        self.ifs_sym = sp.integrate(fs_sym.subs(s, u), (u, 0, s))

    def f(self, t):
        return float(self.fs_sym.subs(self.s, t))

    def F(self, t):
        return float(self.ifs_sym.subs(self.s, t))

    def int4gb(self):
        return float(self._sp.integrate(self.ifs_sym * self.ifs_sym, (self.s, 0, self.T)))


class MyDomain:
    """``MyDomain`` (``DmriFemLib.py:583-637``): mesh + tissue coefficients.

    ``phase`` (per cell, 0/1) or ``mymesh.markers`` select the compartments;
    ``kappa`` is a scalar or an (n_regions, n_regions) array (per-interface
    permeability), constant on each interface facet (``kappa_mode = "facet"``)
    or, with ``kappa_mode = "cr"``, the reference's Crouzeix-Raviart permeability
    field (``MultilayeredDiskVariablePermeability.ipynb:480-502``); ``D`` is a scalar, a per-region array, or a per-cell tensor
    set through :meth:`ImposeDiffusionTensor`.
    """

    def __init__(self, mymesh, mri_para):
        self.mymesh = mymesh
        self.porder = 1
        self.hmin = mymesh.hmin()
        self.hmax = mymesh.hmax()
        self.tol = 1e-2 * self.hmin
        self.gdim = 3
        self.tdim = 3
        lo, hi = mymesh.xyz.min(axis=0), mymesh.xyz.max(axis=0)
        self.xmin, self.ymin, self.zmin = lo
        self.xmax, self.ymax, self.zmax = hi
        self.gdir = mri_para.gdir
        self.qvalue = mri_para.qvalue
        self.phase = None
        self.PeriodicDir = [0, 0, 0]
        self.IsDomainPeriodic = False
        self.IsDomainMultiple = False
        self.kappa = 0.0
        self.kappa_mode = "facet"   # or "cr": the reference's Crouzeix-Raviart permeability field
        self.D = None
        self._D_cell = None
        self.device = 0
        self._ctx = None
        self._state = None

    def ImposeDiffusionTensor(self, k00, k01, k02, k10, k11, k12, k20, k21, k22):
        """Per-cell (or constant) tensor; the symmetric part is used, since the
        engine's COCG needs a complex-symmetric operator."""
        n_t = self.mymesh.num_cells()
        comp = [np.broadcast_to(np.asarray(c, np.float64), (n_t,)) for c in
                (k00, k01, k02, k10, k11, k12, k20, k21, k22)]
        k = np.stack(comp, axis=1).reshape(n_t, 3, 3)
        ks = 0.5 * (k + np.transpose(k, (0, 2, 1)))
        self._D_cell = np.stack([ks[:, 0, 0], ks[:, 1, 1], ks[:, 2, 2], ks[:, 0, 1], ks[:, 0, 2], ks[:, 1, 2]], axis=1)
        self.D = "tensor"

    def Apply(self):
        self._ctx = None

    # -- internal -----------------------------------------------------------
    def regions(self):
        """(cell_region, n_regions, region_compartment)."""
        n_t = self.mymesh.num_cells()
        if self.mymesh.markers is not None and (self.IsDomainMultiple or self.phase is None):
            reg = self.mymesh.markers.astype(np.int32)
        elif self.IsDomainMultiple and self.phase is not None:
            reg = np.rint(np.asarray(self.phase, np.float64)).astype(np.int32)
        else:
            reg = np.zeros(n_t, np.int32)
        if reg.min() < 0:
            raise ValueError("cell markers must be >= 0")
        n_regions = int(reg.max()) + 1
        if self.IsDomainMultiple:
            region_comp = np.arange(n_regions, dtype=np.int32) % 2   # phase = marker % 2
        else:
            region_comp = np.zeros(n_regions, np.int32)
        return reg, n_regions, region_comp

    def context(self, mri_para):
        """Upload + assemble once; re-assemble when coefficients change."""
        reg, nr, rc = self.regions()
        D = self.D if self.D is not None else 3e-3
        # T2: a scalar, one value per region, or one per cell (a DG0 field,
        # T2_Relaxation.ipynb); T2 >= 1e15 means no decay (the reference's 1e16)
        T2a = np.asarray(mri_para.T2, np.float64)
        n_t = self.mymesh.num_cells()
        iT2_cell = None
        if T2a.ndim == 1 and T2a.size == n_t and n_t != nr:
            iT2_cell = np.where(T2a >= 1e15, 0.0, 1.0 / T2a)
            T2a = np.float64(1e16)
        T2 = np.broadcast_to(T2a, (nr,))
        iT2 = np.where(T2 >= 1e15, 0.0, 1.0 / T2)
        kp = np.asarray(self.kappa, np.float64)
        if kp.ndim == 0:
            kp = np.full((nr, nr), float(kp))
        Dr = np.broadcast_to(np.asarray(3e-3 if isinstance(D, str) else D, np.float64), (nr,)).copy()
        key = (Dr.tobytes(), iT2.tobytes(), kp.tobytes(), None if self._D_cell is None else id(self._D_cell),
               None if iT2_cell is None else iT2_cell.tobytes(), self.kappa_mode)
        if self._ctx is None:
            self._ctx = _native.Context(self.device)
            self._ctx.mesh_upload(self.mymesh.xyz, self.mymesh.tets, reg, nr, rc)
            self._state = None
            self._periodic = None
        pdir = tuple(int(bool(d)) for d in self.PeriodicDir)
        mode = "strong" if (self.IsDomainPeriodic and sum(pdir) > 0) else "weak"
        if self._periodic != (pdir, mode):
            self._ctx.set_periodic_mode(mode)
            self._ctx.set_periodic(pdir)
            self._periodic = (pdir, mode)
        if self._state != key:
            self._ctx.set_coefficients(Dr, iT2, kp)
            self._ctx.set_cell_diffusion(self._D_cell)
            self._ctx.set_cell_T2(iT2_cell)
            self._ctx.set_kappa_mode(self.kappa_mode)
            self._ctx.assemble()
            self._state = key
        return self._ctx


class MRI_simulation:
    """``MRI_simulation`` (``DmriFemLib.py:860-915``)."""

    def __init__(self):
        self.nskip = 5
        self.theta = 0.5
        self.k = None
        self.loop = "solve"     # 'solve': while t < T + k ; 'lt_T': while t < T

    def solve(self, mydomain, mri_para, linsolver=None, ic=None):
        """Integrate one signal on the GPU (FP64 by default)."""
        if mri_para.qvalue is None:
            mri_para.Apply()
        ctx = mydomain.context(mri_para)
        mri_para._ensure_profile()
        fn, fo = seqs.profile_samples(mri_para.profile, self.k, self.loop)
        ctx.set_schedule(fn, fo, self.k, self.theta)
        if sum(mydomain.PeriodicDir) > 0:
            ctx.set_schedule_integral(*seqs.integral_samples(mri_para.profile, self.k, self.loop))
        params = getattr(linsolver, "parameters", {}) if linsolver is not None else {}
        rtol = float(params.get("relative_tolerance", 1e-12))
        maxit = int(params.get("maximum_iterations", 2000))
        prec = _native.PRECISION_MIXED if params.get("precision", "fp64") == "mixed" else _native.PRECISION_FP64
        u0 = None if ic is None else np.asarray(ic, np.float64)
        t0 = time.time()
        out = ctx.solve(mri_para.qvalue, mri_para.gdir, None, u0, prec, rtol, min(maxit, 2 ** 31 - 1),
                        compartments=True)
        self.elapsed_time = time.time() - t0
        self.signal = float(out["signal"][0])
        self.compartment_signals = out["compartments"][0].tolist()
        self.voi = out["S0"]
        self.whole_vol = ctx.info()["volume"]
        self.stats = out["stats"]
        self.u_0 = ctx.solution(0)
        self.Dirac_Delta = ic
        self.t = (len(fn)) * self.k
        self.nsteps = len(fn)
        return self.signal


def simulate(mydomain, profiles, bvalues, gdirs, profile_index=None, k=200.0, theta=0.5,
             precision="fp64", rtol=None, max_iterations=2000, ic=None, T2=1e16, loop="solve"):
    """Many signals on one domain in one engine call: bvalues[n], gdirs[n,3],
    profile_index[n] into ``profiles``.  Returns (signals/S0, raw dict)."""
    profiles = list(profiles)
    bvalues = np.asarray(bvalues, np.float64)
    n = len(bvalues)
    gd = np.asarray(gdirs, np.float64).reshape(n, 3)
    gd = gd / np.linalg.norm(gd, axis=1, keepdims=True)
    pidx = np.zeros(n, np.int32) if profile_index is None else np.asarray(profile_index, np.int32)
    steps = None
    fns, fos, int4 = [], [], []
    for p in profiles:
        fn, fo = seqs.profile_samples(p, k, loop)
        if steps is None:
            steps = len(fn)
        if len(fn) != steps:
            raise ValueError("all profiles in one call must have the same number of steps")
        fns.append(fn)
        fos.append(fo)
        int4.append(p.int4gb())
    q = np.array([seqs.b_to_q(b, int4[i]) for b, i in zip(bvalues, pidx)])
    para = MRI_parameters()
    para.T2 = T2
    ctx = mydomain.context(para)
    ctx.set_schedule(np.array(fns), np.array(fos), k, theta)
    if sum(mydomain.PeriodicDir) > 0:
        Fs = [seqs.integral_samples(p, k, loop) for p in profiles]
        ctx.set_schedule_integral(np.array([f[0] for f in Fs]), np.array([f[1] for f in Fs]))
    prec = _native.PRECISION_MIXED if precision == "mixed" else _native.PRECISION_FP64
    if rtol is None:
        rtol = 1e-12 if prec == _native.PRECISION_FP64 else 1e-9
    out = ctx.solve(q, gd, pidx, ic, prec, rtol, max_iterations, compartments=True)
    return out["signal"] / out["S0"], out


def PostProcessing(mydomain, mri_para, mri_simu, plt=None, ms="", logfile="log.txt"):
    """Signal report of ``PostProcessing`` (``DmriFemLib.py:917-988``): prints
    the reference's result line and appends it to ``log.txt``."""
    voi = mri_simu.voi
    signal = mri_simu.signal
    whole_vol = mri_simu.whole_vol
    if mydomain.IsDomainMultiple:
        s0, s1 = (mri_simu.compartment_signals + [0.0, 0.0])[:2]
        kap = mydomain.kappa
        if np.isscalar(kap):
            out_text = ('b: %.3f, g: %.3f, q: %.3e, Signal: %.3e, Normalized signal: %.6e, kappa: %.3e, '
                        'dt: %.3f, hmin: %.3e, hmax: %.3e, whole_vol: %.3f, vol_of_interest: %.3f, '
                        'elasped time %.3f (s)\n' % (mri_para.bvalue, mri_para.gvalue, mri_para.qvalue, signal,
                                                    signal / voi, kap, mri_simu.k, mydomain.hmin, mydomain.hmax,
                                                    whole_vol, voi, mri_simu.elapsed_time))
        else:
            out_text = ('b: %.3f, g: %.3f, q: %.3e, Signal: %.3e, Normalized signal: %.6e, dt: %.3f, '
                        'hmin: %.3e, hmax: %.3e, whole_vol: %.3f, vol_of_interest: %.3f, elasped time %.3f (s)\n'
                        % (mri_para.bvalue, mri_para.gvalue, mri_para.qvalue, signal, signal / voi, mri_simu.k,
                           mydomain.hmin, mydomain.hmax, whole_vol, voi, mri_simu.elapsed_time))
        print("Signal on each compartment")
        print("Signal0: %.3e" % s0)
        print("Signal1: %.3e" % s1)
    else:
        out_text = ('b: %.3f, g: %.3f, q: %.3e, Signal: %.3e, Normalized signal: %.6e, dt: %.3f, hmin: %.3e, '
                    'hmax: %.3e, whole_vol: %.3f, vol_of_interest: %.3f, elasped time %.3f (s)\n'
                    % (mri_para.bvalue, mri_para.gvalue, mri_para.qvalue, signal, signal / voi, mri_simu.k,
                       mydomain.hmin, mydomain.hmax, whole_vol, voi, mri_simu.elapsed_time))
    print(out_text, end="")
    if logfile:
        with open(logfile, "a") as fh:
            if ms:
                fh.write("%" + ms + "\n")
            fh.write(out_text)
    return out_text
