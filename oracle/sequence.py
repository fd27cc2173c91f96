"""Gradient time profiles and the b -> q conversion -- TEST INFRASTRUCTURE ONLY.

Restates ``MRI_parameters`` (``DmriFemLib.py:800-858``) without sympy (sympy is
not available on every machine the oracle runs on):

* ``time_profile``   (``DmriFemLib.py:834-835``): f(t) from a sympy
  ``Piecewise`` -- first branch whose condition holds wins.  The PGSE branches
  are ``GCloudDmriSolver.py:188-193``, cos-OGSE ``ArbitraryTimeSequence.ipynb:380-392``.
* ``itime_profile_sym`` (``DmriFemLib.py:829-832``): F(s) = int_0^s f.
* ``integral_term_for_gb`` (``DmriFemLib.py:826-827``): int4gb = int_0^T F(s)^2 ds.
* ``convert_b2q`` (``DmriFemLib.py:840-842``): q = sqrt(b) / sqrt(int4gb).

sympy integrates symbolically; here each piece is integrated with 48-point
Gauss-Legendre (exact for the polynomial pieces, and below 1e-15 relative for
one cosine period per piece).  ``tests/test_oracle_pins.py`` checks this
against sympy on the reference's own Piecewise expressions.
"""

import math
import numpy as np

_GL_X, _GL_W = np.polynomial.legendre.leggauss(48)


class Sequence:
    """Piecewise gradient profile.

    ``pieces`` is a list of ``(bound, inclusive, fn)``: f(s) = fn(s) for the
    first piece with ``s < bound`` (``s <= bound`` when inclusive); after the
    last piece f = 0, like the reference's trailing ``(0., True)`` branch.
    ``fn`` must accept numpy arrays.  ``T`` is the echo time.
    """

    def __init__(self, pieces, T, name="custom"):
        self.pieces = list(pieces)
        self.T = float(T)
        self.name = name
        bps = sorted({0.0} | {float(b) for b, _, _ in self.pieces if b > 0.0})
        self._bps = bps

    def _fn_at(self, s):
        for bound, inclusive, fn in self.pieces:
            if (s <= bound) if inclusive else (s < bound):
                return fn
        return None

    def f(self, s):
        fn = self._fn_at(s)
        return 0.0 if fn is None else float(fn(np.float64(s)))

    def _intervals(self, upto):
        """Intervals [a,b] between breakpoints covering [0, upto], each with the
        piece active in its interior (boundary semantics do not matter for
        integrals)."""
        out = []
        pts = [b for b in self._bps if b < upto] + [upto]
        for a, b in zip(pts[:-1], pts[1:]):
            if b > a:
                out.append((a, b, self._fn_at(0.5 * (a + b))))
        return out

    @staticmethod
    def _gl(fun, a, b):
        x = 0.5 * (b - a) * _GL_X + 0.5 * (b + a)
        return 0.5 * (b - a) * float(np.dot(_GL_W, fun(x)))

    def F(self, s):
        """int_0^s f(u) du (``itime_profile``)."""
        total = 0.0
        for a, b, fn in self._intervals(float(s)):
            if fn is not None:
                total += self._gl(fn, a, b)
        return total

    def int4gb(self):
        """int_0^T F(s)^2 ds (``integral_term_for_gb``)."""
        total = 0.0
        for a, b, _ in self._intervals(self.T):
            total += self._gl(lambda x: np.array([self.F(v) ** 2 for v in x]), a, b)
        return total


def _const(c):
    return lambda s: np.full(np.shape(s), c, dtype=np.float64)


def PGSE(delta, Delta):
    """Pulsed-gradient spin echo, ``GCloudDmriSolver.py:186-193``."""
    delta = float(delta)
    Delta = float(Delta)
    T = Delta + delta
    return Sequence([
        (delta, False, _const(1.0)),
        (Delta, False, _const(0.0)),
        (T, False, _const(-1.0)),
    ], T, name="PGSE")


def CosOGSE(delta, Delta, nperiod=1, t0=0.0, seq_ext=0.0):
    """cos-OGSE, ``ArbitraryTimeSequence.ipynb:380-392`` (profile 3).

    omega = 2 pi nperiod / delta, second lobe at tau = (Delta+delta)/2,
    T = Delta + delta + t0 + seq_ext.
    """
    delta = float(delta)
    Delta = float(Delta)
    Dd = Delta + delta
    T = Dd + t0 + seq_ext
    omega = 2.0 * nperiod * math.pi / delta
    tau = Dd / 2.0
    return Sequence([
        (t0, False, _const(0.0)),
        (delta + t0, True, lambda s: np.cos(omega * (s - t0))),
        (tau + t0, True, _const(0.0)),
        (delta + tau + t0, True, lambda s: -np.cos(omega * (s - t0 - tau))),
    ], T, name="cos-OGSE")


def bvalue_to_q(bvalue, int4gb):
    """``convert_b2q`` (``DmriFemLib.py:840-842``)."""
    return math.sqrt(bvalue) / math.sqrt(int4gb)


def q_to_g(q):
    """``convert_q2g`` (``DmriFemLib.py:683-686``), gamma = 2.675e8, for printing only."""
    return q / 2.675e8 * 1e12


def reference_schedule(T, k, loop="solve"):
    """(t_new, t_old) of every solve, replaying the reference's float loop.

    ``loop='solve'``: ``MRI_simulation.solve`` (``DmriFemLib.py:886-911``):
    t = tp = 0; while t < T + k: solve with f(t) implicit, f(tp) explicit;
    tp = t; t += k.
    ``loop='lt_T'``: the inlined loop of ``ConvergenceTest.ipynb:366-395``
    (``while t < T``, same lag).
    """
    t = 0.0
    tp = 0.0
    new, old = [], []
    end = T + k if loop == "solve" else T
    while t < end:
        new.append(t)
        old.append(tp)
        tp = t
        t += k
    return np.array(new), np.array(old)
