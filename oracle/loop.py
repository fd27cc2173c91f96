"""Crank-Nicolson time loop and signal -- TEST INFRASTRUCTURE ONLY.

Restates ``MRI_simulation.solve`` (``DmriFemLib.py:878-915``) and the signal of
``PostProcessing`` (``DmriFemLib.py:917-931``):

* the initial condition is the P1 interpolant of ``|x|^2 < 1e6`` (= 1 on every
  vertex of the meshes used here) in u0r and, for two compartments, u1r
  (``DmriFemLib.py:865-876``);
* every step solves ``(1/k) M + assemble(F(f(t)))`` against
  ``assemble(L(u_old, f(t_prev)))`` (``DmriFemLib.py:901-907``) on the
  schedule of ``sequence.reference_schedule``;
* the signal is ``int (phase u1r + (1-phase) u0r) dx`` and the normalisation
  ``voi = int Dirac_Delta dx`` (``DmriFemLib.py:922-931``).

Linear solvers: ``'lu'`` is the reference's ``PETScLUSolver("mumps")``
alternative (``GCloudDmriSolver.py:218``; ``ConvergenceTest.ipynb:353``) via
SuperLU, factorised once per distinct implicit f value (the matrix depends on
the step only through f(t), so PGSE needs three factorisations);
``'bicgstab'`` is the shipped ``KrylovSolver("bicgstab", "jacobi")`` with
rtol 1e-9 / atol 1e-10 from a zero initial guess (``GCloudDmriSolver.py:219-222``).
"""

import time
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sps
import scipy.sparse.linalg as spla

from .sequence import reference_schedule


@dataclass
class OracleResult:
    signal: float
    S0: float
    normalized: float
    compartment_signals: list = field(default_factory=list)
    u: np.ndarray = None
    steps: int = 0
    elapsed: float = 0.0
    iterations: list = field(default_factory=list)


def _schedule_f(seq, k, loop):
    tn, to = reference_schedule(seq.T, k, loop)
    return np.array([seq.f(t) for t in tn]), np.array([seq.f(t) for t in to])


def _jacobi_bicgstab(A, b, rtol, atol, maxiter):
    d = A.diagonal()
    P = spla.LinearOperator(A.shape, matvec=lambda v: v / d, dtype=A.dtype)
    it = [0]

    def cb(_):
        it[0] += 1
    x, info = spla.bicgstab(A, b, rtol=rtol, atol=atol, maxiter=maxiter, M=P, callback=cb)
    if info != 0:
        raise RuntimeError("BiCGSTAB did not converge (info=%d)" % info)
    return x, it[0]


def solve_duplicated(sysd, seq, q, gdir, k, theta=0.5, loop="solve", u0=None,
                     solver="lu", rtol=1e-9, atol=1e-10, max_steps=None, periodic=None):
    """Time loop on the complex duplicated-node system of ``forms.duplicated_system``.

    ``q`` is ``mri_para.qvalue``; ``gdir`` is normalised as in
    ``set_gradient_dir`` (``DmriFemLib.py:809-824``).  ``max_steps`` truncates
    the loop (bounded CPU-timing samples only).  ``periodic`` is the output of
    ``periodic.weak_periodic``: the implicit matrix gains theta B and every
    right-hand side (1 - theta) B ubc(u_n, F(tp)) (``DmriFemLib.py:58-145``).
    """
    g = np.asarray(gdir, dtype=np.float64)
    g = g / np.linalg.norm(g)
    n = sysd["n"]
    M, S = sysd["M"], (sysd["K"] + sysd["T"] + sysd["R"]).tocsr()
    Jg = (g[0] * sysd["Jx"] + g[1] * sysd["Jy"] + g[2] * sysd["Jz"]).tocsr()
    Mk = (1.0 / k) * M
    f_new, f_old = _schedule_f(seq, k, loop)
    if max_steps is not None:
        f_new, f_old = f_new[:max_steps], f_old[:max_steps]
    n_v = len(sysd["vertex_weight"])
    ic = np.ones(n_v) if u0 is None else np.asarray(u0, dtype=np.float64)
    u = ic[sysd["vertex"]].astype(np.complex128)
    S0 = float(np.dot(sysd["vertex_weight"], ic))
    Abase = (Mk + theta * S).astype(np.complex128).tocsc()
    Bbase = (Mk - (1.0 - theta) * S).astype(np.complex128).tocsr()
    if periodic is not None:
        from .periodic import ubc
        Abase = (Abase + theta * periodic["B"].astype(np.complex128)).tocsc()
        Bper = periodic["B"].astype(np.complex128).tocsr()
        _, t_old = reference_schedule(seq.T, k, loop)
        F_old = np.array([seq.F(t) for t in t_old])[:len(f_old)]
    Jc = Jg.astype(np.complex128)
    cache = {}
    iters = []
    t0 = time.perf_counter()
    for step, (fn, fo) in enumerate(zip(f_new, f_old)):
        rhs = Bbase @ u - 1j * ((1.0 - theta) * q * fo) * (Jc @ u)
        if periodic is not None:
            rhs = rhs + (1.0 - theta) * (Bper @ ubc(periodic, u, q, g, F_old[step]))
        A = (Abase + 1j * (theta * q * fn) * Jc.tocsc())
        if solver == "lu":
            lu = cache.get(fn)
            if lu is None:
                lu = spla.splu(A.tocsc())
                cache[fn] = lu
            u = lu.solve(rhs)
        elif solver == "bicgstab":
            u, it = _jacobi_bicgstab(A.tocsr(), rhs, rtol, atol, 100000)
            iters.append(it)
        else:
            raise ValueError(solver)
    elapsed = time.perf_counter() - t0
    w = sysd["w"]
    sig = float(np.dot(w, u.real))
    comp = [float(np.dot(w[sysd["field"] == f], u.real[sysd["field"] == f]))
            for f in range(sysd["n_fields"])]
    return OracleResult(sig, S0, sig / S0, comp, u, len(f_new), elapsed, iters)


def solve_two_field(sys2, seq, q, gdir, k, theta=0.5, loop="solve", u0=None,
                    solver="lu", rtol=1e-9, atol=1e-10, max_steps=None):
    """Time loop on the literal real mixed system of ``forms.two_field_system``."""
    g = np.asarray(gdir, dtype=np.float64)
    g = g / np.linalg.norm(g)
    n_v, nf = sys2["n_v"], sys2["nf"]
    Jg = (g[0] * sys2["Jfuncs"][0] + g[1] * sys2["Jfuncs"][1] + g[2] * sys2["Jfuncs"][2]).tocsr()
    S = sys2["S"]
    f_new, f_old = _schedule_f(seq, k, loop)
    if max_steps is not None:
        f_new, f_old = f_new[:max_steps], f_old[:max_steps]
    ic = np.ones(n_v) if u0 is None else np.asarray(u0, dtype=np.float64)
    u = np.zeros(sys2["N"])
    for f in range(nf):
        u[2 * f * n_v:(2 * f + 1) * n_v] = ic          # assign(u_0.sub(0|2), Dirac_Delta)
    S0 = float(np.dot(sys2["vertex_weight"], ic))
    Amass = (1.0 / k) * sys2["Mid"]
    Lmass = (1.0 / k) * sys2["Mz"]
    cache = {}
    iters = []
    t0 = time.perf_counter()
    for fn, fo in zip(f_new, f_old):
        # F = -theta FuncF + theta*interface ; L = u/k + (1-theta) FuncF - (1-theta) interface
        A = (Amass + theta * S - (theta * fn * q) * Jg)
        b = Lmass @ u + ((1.0 - theta) * fo * q) * (Jg @ u) - (1.0 - theta) * (S @ u)
        if solver == "lu":
            lu = cache.get(fn)
            if lu is None:
                lu = spla.splu(sps.csc_matrix(A))
                cache[fn] = lu
            u = lu.solve(b)
        elif solver == "bicgstab":
            u, it = _jacobi_bicgstab(A.tocsr(), b, rtol, atol, 100000)
            iters.append(it)
        else:
            raise ValueError(solver)
    elapsed = time.perf_counter() - t0
    comp = [float(np.dot(sys2["w_comp"][f], u[2 * f * n_v:(2 * f + 1) * n_v])) for f in range(nf)]
    sig = float(sum(comp))
    return OracleResult(sig, S0, sig / S0, comp, u, len(f_new), elapsed, iters)
