"""Diffusion-encoding time profiles f(t), the b <-> q conversion and the
reference's time-step schedule.

Mirrors ``MRI_parameters`` of the reference (``DmriFemLib.py:800-858``):
``time_profile`` evaluates f(t) with the branch semantics of a sympy
``Piecewise`` (first true condition wins, strict ``<`` or inclusive ``<=`` per
branch), ``integral_term_for_gb`` is int_0^T (int_0^s f)^2 ds and
``convert_b2q`` is q = sqrt(b) / sqrt(int4gb).  The profiles are the ones of
``GCloudDmriSolver.py:188-193`` (PGSE) and ``ArbitraryTimeSequence.ipynb:348-449``
(profiles 1-6).  No sympy: constant and linear segments are integrated in
closed form, trigonometric ones with 64-point Gauss-Legendre per segment.
"""

import math

import numpy as np

GAMMA = 2.675e8  # rad/s/T as in convert_g2q / convert_q2g (DmriFemLib.py:680-686)

_GLX, _GLW = np.polynomial.legendre.leggauss(64)


class Segment:
    """f(s) on one branch: ``kind`` 'poly' (c0 + c1 (s - s0)), 'cos' or 'sin'
    (amp * cos|sin(omega (s - s0)))."""

    __slots__ = ("end", "inclusive", "kind", "a", "b", "s0")

    def __init__(self, end, inclusive, kind, a=0.0, b=0.0, s0=0.0):
        self.end = float(end)
        self.inclusive = bool(inclusive)
        self.kind = kind
        self.a = float(a)   # poly: c0 ; trig: amplitude
        self.b = float(b)   # poly: c1 ; trig: omega
        self.s0 = float(s0)

    def value(self, s):
        if self.kind == "poly":
            return self.a + self.b * (s - self.s0)
        if self.kind == "cos":
            return self.a * np.cos(self.b * (s - self.s0))
        return self.a * np.sin(self.b * (s - self.s0))

    def holds(self, s):
        return s <= self.end if self.inclusive else s < self.end


class TimeProfile:
    """A piecewise gradient profile with echo time ``T``."""

    def __init__(self, segments, T, name="custom"):
        self.segments = list(segments)
        self.T = float(T)
        self.name = name
        cuts = {0.0, self.T}
        for sg in self.segments:
            if 0.0 < sg.end < self.T:
                cuts.add(sg.end)
        self._cuts = sorted(cuts)
        self._F_at_cut = None

    # -- f(t) exactly as the reference's Piecewise evaluates it
    def f(self, t):
        for sg in self.segments:
            if sg.holds(t):
                return float(sg.value(np.float64(t)))
        return 0.0

    def _active(self, a, b):
        mid = 0.5 * (a + b)
        for sg in self.segments:
            if sg.holds(mid):
                return sg
        return None

    @staticmethod
    def _seg_integral(sg, a, b):
        """int_a^b f and int_a^b (int_a^s f)^2 ds on one segment."""
        L = b - a
        if sg is None:
            return 0.0, 0.0
        if sg.kind == "poly":
            p0 = sg.a + sg.b * (a - sg.s0)   # value at a
            p1 = sg.b
            I = p0 * L + 0.5 * p1 * L * L
            I2 = p0 * p0 * L ** 3 / 3.0 + p0 * p1 * L ** 4 / 4.0 + p1 * p1 * L ** 5 / 20.0
            return I, I2
        x = 0.5 * L * _GLX + 0.5 * (a + b)
        w = 0.5 * L * _GLW
        I = float(np.dot(w, sg.value(x)))
        # G(s) = int_a^s f: closed form for trig segments
        if sg.kind == "cos":
            G = sg.a / sg.b * (np.sin(sg.b * (x - sg.s0)) - math.sin(sg.b * (a - sg.s0)))
        else:
            G = -sg.a / sg.b * (np.cos(sg.b * (x - sg.s0)) - math.cos(sg.b * (a - sg.s0)))
        return I, G

    def F(self, t):
        """int_0^t f (``itime_profile``)."""
        total = 0.0
        for a, b in zip(self._cuts[:-1], self._cuts[1:]):
            if t <= a:
                break
            hi = min(t, b)
            I, _ = self._seg_integral(self._active(a, b), a, hi)
            total += I
        if t > self._cuts[-1]:
            I, _ = self._seg_integral(self._active(self._cuts[-1], t), self._cuts[-1], t)
            total += I
        return total

    def int4gb(self):
        """int_0^T F(s)^2 ds (``integral_term_for_gb``)."""
        total = 0.0
        Fa = 0.0
        for a, b in zip(self._cuts[:-1], self._cuts[1:]):
            sg = self._active(a, b)
            L = b - a
            I, G = self._seg_integral(sg, a, b)
            if sg is None or sg.kind == "poly":
                # int (Fa + G)^2 = Fa^2 L + 2 Fa int G + int G^2
                if sg is None:
                    intG, intG2 = 0.0, 0.0
                else:
                    p0 = sg.a + sg.b * (a - sg.s0)
                    p1 = sg.b
                    intG = p0 * L * L / 2.0 + p1 * L ** 3 / 6.0
                    intG2 = G
                total += Fa * Fa * L + 2.0 * Fa * intG + intG2
            else:
                w = 0.5 * L * _GLW
                total += float(np.dot(w, (Fa + G) ** 2))
            Fa += I
        return total


def pgse(delta, Delta, t0=0.0, seq_ext=0.0):
    """PGSE (``GCloudDmriSolver.py:188-193``; with t0/seq_ext, profile 1 of
    ``ArbitraryTimeSequence.ipynb:348-358``)."""
    d, D = float(delta), float(Delta)
    segs = []
    if t0 > 0:
        segs.append(Segment(t0, False, "poly", 0.0))
    segs += [Segment(d + t0, False, "poly", 1.0), Segment(D + t0, False, "poly", 0.0),
             Segment(D + d + t0, False, "poly", -1.0)]
    return TimeProfile(segs, D + d + t0 + seq_ext, "PGSE")


def double_pgse(delta, Delta, t0=0.0, seq_ext=0.0):
    """Profile 2 of ``ArbitraryTimeSequence.ipynb:360-376``."""
    d, D = float(delta), float(Delta)
    Dd = D + d
    disp = Dd + d
    segs = [Segment(t0, False, "poly", 0.0), Segment(d + t0, False, "poly", 1.0),
            Segment(D + t0, False, "poly", 0.0), Segment(Dd + t0, False, "poly", -1.0),
            Segment(disp, False, "poly", 0.0), Segment(t0 + disp, False, "poly", 0.0),
            Segment(d + t0 + disp, False, "poly", 1.0), Segment(D + t0 + disp, False, "poly", 0.0),
            Segment(Dd + t0 + disp, False, "poly", -1.0)]
    return TimeProfile(segs, 2 * Dd + t0 + d + seq_ext, "Double PGSE")


def cos_ogse(delta, Delta, nperiod=1, t0=0.0, seq_ext=0.0):
    """cos-OGSE, profile 3 of ``ArbitraryTimeSequence.ipynb:378-392``:
    omega = 2 pi n / delta, second lobe at tau = (Delta + delta) / 2."""
    d, D = float(delta), float(Delta)
    Dd = D + d
    om = 2.0 * nperiod * math.pi / d
    tau = Dd / 2.0
    segs = [Segment(t0, False, "poly", 0.0), Segment(d + t0, True, "cos", 1.0, om, t0),
            Segment(tau + t0, True, "poly", 0.0), Segment(d + tau + t0, True, "cos", -1.0, om, t0 + tau)]
    return TimeProfile(segs, Dd + t0 + seq_ext, "cos-OGSE")


def sin_ogse(delta, Delta, nperiod=1, t0=0.0, seq_ext=0.0):
    """sin-OGSE, profile 4 of ``ArbitraryTimeSequence.ipynb:393-406``."""
    d, D = float(delta), float(Delta)
    Dd = D + d
    om = 2.0 * nperiod * math.pi / d
    tau = Dd / 2.0
    segs = [Segment(t0, False, "poly", 0.0), Segment(d + t0, True, "sin", 1.0, om, t0),
            Segment(tau + t0, True, "poly", 0.0), Segment(d + tau + t0, True, "sin", -1.0, om, t0 + tau)]
    return TimeProfile(segs, Dd + t0 + seq_ext, "sin-OGSE")


def trapezoid_pgse(delta, Delta, t0=0.0, seq_ext=0.0):
    """Trapezoid PGSE with rise time delta/3, profile 5 of
    ``ArbitraryTimeSequence.ipynb:407-420``."""
    d, D = float(delta), float(Delta)
    Dd = D + d
    tau = d / 3.0
    segs = [Segment(t0, False, "poly", 0.0),
            Segment(tau + t0, False, "poly", 0.0, 1.0 / tau, t0),
            Segment(d - tau + t0, False, "poly", 1.0),
            Segment(d + t0, False, "poly", 0.0, -1.0 / tau, t0 + d),
            Segment(D + t0, False, "poly", 0.0),
            Segment(D + tau + t0, False, "poly", 0.0, -1.0 / tau, t0 + D),
            Segment(Dd - tau + t0, False, "poly", -1.0),
            Segment(Dd + t0, False, "poly", 0.0, 1.0 / tau, t0 + Dd)]
    return TimeProfile(segs, Dd + t0 + seq_ext, "Trapezoid PGSE")


def schedule(T, k, loop="solve"):
    """(t_new, t_old) of every solve of the reference's loop.

    ``MRI_simulation.solve`` (``DmriFemLib.py:886-911``) starts at t = tp = 0,
    runs ``while t < T + k`` and evaluates f(t) in the implicit form and f(tp)
    in the explicit one before ``tp = t; t += k``.  ``loop='lt_T'`` is the
    ``while t < T`` variant inlined in ``ConvergenceTest.ipynb:366-395``.
    """
    end = T + k if loop == "solve" else T
    t, tp = 0.0, 0.0
    tn, to = [], []
    while t < end:
        tn.append(t)
        to.append(tp)
        tp = t
        t += k
    return np.asarray(tn), np.asarray(to)


def profile_samples(profile, k, loop="solve"):
    """f at the implicit and explicit level of every step."""
    tn, to = schedule(profile.T, k, loop)
    return (np.array([profile.f(t) for t in tn]), np.array([profile.f(t) for t in to]))


def phase_samples(profile, k, loop="solve"):
    """F(tp) = int_0^tp f at the explicit level of every step: the phase of the
    pseudo-periodic boundary term (``itime_profile(tp)`` handed to
    ``WeakPseudoPeriodic.set_values``, ``DmriFemLib.py:73, 117, 901-905``)."""
    _, to = schedule(profile.T, k, loop)
    return np.array([profile.F(t) for t in to])


def integral_samples(profile, k, loop="solve"):
    """ift = int_0^t f at the implicit and explicit level of every step: the
    ``itime_profile(t)`` and ``itime_profile(tp)`` of the strong pseudo-periodic
    forms (``DmriFemLib.py:148-238, 897-905``)."""
    tn, to = schedule(profile.T, k, loop)
    return np.array([profile.F(t) for t in tn]), np.array([profile.F(t) for t in to])


def b_to_q(bvalue, int4gb):
    """``convert_b2q`` (``DmriFemLib.py:840-842``)."""
    return math.sqrt(bvalue) / math.sqrt(int4gb)


def q_to_b(q, int4gb):
    return q * q * int4gb


def q_to_g(q):
    """``convert_q2g`` (``DmriFemLib.py:683-686``)."""
    return q / GAMMA * 1e12


def g_to_q(g):
    """``convert_g2q`` (``DmriFemLib.py:679-681``)."""
    return g * GAMMA * 1e-12
