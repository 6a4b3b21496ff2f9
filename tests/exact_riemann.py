"""Exact solutions of the 1-D Riemann problem, for the oracle's shock-tube
tests (test infrastructure, written from the published methods):

- Newtonian ideal gas: the pressure function of Toro, *Riemann Solvers and
  Numerical Methods for Fluid Dynamics*, ch. 4 (shock branch from the
  Rankine-Hugoniot conditions, rarefaction branch from the isentropic
  Riemann invariants), solved for the star pressure by bisection and sampled
  along x/t.
- Special-relativistic ideal gas with no tangential velocity: Marti & Muller,
  J. Fluid Mech. 258 (1994) 317, and their Living Review (2003): across a
  rarefaction the invariant 1/2 ln((1+v)/(1-v)) +- 1/sqrt(g-1)
  ln((sqrt(g-1)+c)/(sqrt(g-1)-c)) is constant on the isentrope; across a
  shock the Taub adiabat gives the post-shock enthalpy, the mass flux j and
  the shock velocity, and the post-shock velocity follows. The star pressure
  is found by bisection on v*_L(p) = v*_R(p).

States are (rho, v, p): rest-mass density, velocity along x (a 3-velocity in
units of c for SRHD), pressure (in units of rho c^2 for SRHD).
"""
import math

import numpy as np


def _bisect(f, lo, hi, iters=200):
    flo = f(lo)
    for _ in range(iters):
        mid = math.sqrt(lo * hi) if lo > 0 and hi / lo > 4 else 0.5 * (lo + hi)
        fm = f(mid)
        if (fm > 0) == (flo > 0):
            lo, flo = mid, fm
        else:
            hi = mid
        if hi - lo <= 1e-15 * hi:
            break
    return 0.5 * (lo + hi)


# ---------------------------------------------------------------- Newtonian
class Newtonian:
    def __init__(self, left, right, gamma):
        self.g = g = gamma
        self.L, self.R = left, right
        rl, ul, pl = left
        rr, ur, pr = right
        self.cl, self.cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)

        def f(p, rho, pk, ck):
            if p > pk:   # shock
                A, B = 2.0 / ((g + 1.0) * rho), (g - 1.0) / (g + 1.0) * pk
                return (p - pk) * math.sqrt(A / (p + B))
            return 2.0 * ck / (g - 1.0) * ((p / pk) ** ((g - 1.0) / (2.0 * g)) - 1.0)

        self._f = f
        F = lambda p: f(p, rl, pl, self.cl) + f(p, rr, pr, self.cr) + (ur - ul)
        self.ps = _bisect(F, 1e-12 * min(pl, pr), 1e3 * max(pl, pr))
        self.us = 0.5 * (ul + ur) + 0.5 * (f(self.ps, rr, pr, self.cr) - f(self.ps, rl, pl, self.cl))

    def sample(self, xi):
        g, ps, us = self.g, self.ps, self.us
        gm = (g - 1.0) / (g + 1.0)
        if xi <= us:
            rho, u, p, c, s = *self.L, self.cl, -1.0
        else:
            rho, u, p, c, s = *self.R, self.cr, 1.0
        if ps > p:   # shock
            S = u + s * c * math.sqrt((g + 1.0) / (2.0 * g) * ps / p + (g - 1.0) / (2.0 * g))
            if s * (xi - S) >= 0:
                return rho, u, p
            return rho * (ps / p + gm) / (gm * ps / p + 1.0), us, ps
        head = u + s * c
        if s * (xi - head) >= 0:
            return rho, u, p
        cs = c * (ps / p) ** ((g - 1.0) / (2.0 * g))
        tail = us + s * cs
        if s * (xi - tail) <= 0:
            return rho * (ps / p) ** (1.0 / g), us, ps
        uf = 2.0 / (g + 1.0) * (-s * c + 0.5 * (g - 1.0) * u + xi)
        cf = 2.0 / (g + 1.0) * (c - s * 0.5 * (g - 1.0) * (u - xi))
        return rho * (cf / c) ** (2.0 / (g - 1.0)), uf, p * (cf / c) ** (2.0 * g / (g - 1.0))


# ---------------------------------------------------------------------- SRHD
def _h(g, rho, p):
    return 1.0 + g / (g - 1.0) * p / rho


def _cs(g, rho, p):
    return math.sqrt(g * p / (rho * _h(g, rho, p)))


def srhd_conserved(g, rho, v, p):
    """(D, S, tau) and their fluxes (D v, S v + p, S - D v)."""
    W = 1.0 / math.sqrt(1.0 - v * v)
    h = _h(g, rho, p)
    D, S = rho * W, rho * h * W * W * v
    tau = rho * h * W * W - p - D
    return np.array([D, S, tau]), np.array([D * v, S * v + p, S - D * v])


class Relativistic:
    def __init__(self, left, right, gamma):
        self.g = g = gamma
        self.L, self.R = left, right
        F = lambda p: self.v_after(self.L, p, -1.0) - self.v_after(self.R, p, 1.0)
        self.ps = _bisect(lambda p: -F(p), 1e-12 * min(left[2], right[2]), 1e3 * max(left[2], right[2]))
        self.vs = self.v_after(self.L, self.ps, -1.0)

    def rarefaction(self, a, p, s):
        """State on the isentrope of a at pressure p, reached through a wave
        of family s (-1 left-facing, +1 right-facing)."""
        g = self.g
        rho_a, v_a, p_a = a
        rho = rho_a * (p / p_a) ** (1.0 / g)
        sg = math.sqrt(g - 1.0)
        c, ca = _cs(g, rho, p), _cs(g, rho_a, p_a)
        A = ((sg - c) / (sg + c) * (sg + ca) / (sg - ca)) ** (-s * 2.0 / sg)
        v = ((1.0 + v_a) * A - (1.0 - v_a)) / ((1.0 + v_a) * A + (1.0 - v_a))
        return rho, v

    def shock(self, a, p, s):
        """Post-shock (rho, v) and shock velocity for a shock of family s
        into state a with post-shock pressure p > p_a."""
        g = self.g
        rho_a, v_a, p_a = a
        h_a = _h(g, rho_a, p_a)
        dp = p - p_a
        k = (g - 1.0) * dp / (g * p)
        c0 = h_a * h_a + h_a * dp / rho_a
        h_b = (-k + math.sqrt(k * k + 4.0 * (1.0 - k) * c0)) / (2.0 * (1.0 - k))
        rho_b = g * p / ((g - 1.0) * (h_b - 1.0))
        j = s * math.sqrt(dp / (h_a / rho_a - h_b / rho_b))
        Wa = 1.0 / math.sqrt(1.0 - v_a * v_a)
        r2 = rho_a * rho_a * Wa * Wa
        Vs = (r2 * v_a + s * abs(j) * math.sqrt(j * j + r2 * (1.0 - v_a * v_a))) / (r2 + j * j)
        Ws = 1.0 / math.sqrt(1.0 - Vs * Vs)
        v_b = (h_a * Wa * v_a + Ws * dp / j) / (h_a * Wa + dp * (Ws * v_a / j + 1.0 / (rho_a * Wa)))
        return rho_b, v_b, Vs

    def v_after(self, a, p, s):
        if p > a[2]:
            return self.shock(a, p, s)[1]
        return self.rarefaction(a, p, s)[1]

    def sample(self, xi):
        g, ps, vs = self.g, self.ps, self.vs
        a, s = (self.L, -1.0) if xi <= vs else (self.R, 1.0)
        rho_a, v_a, p_a = a
        if ps > p_a:
            rho_b, _, Vs = self.shock(a, ps, s)
            if s * (xi - Vs) >= 0:
                return rho_a, v_a, p_a
            return rho_b, vs, ps

        def speed(rho, v, p):
            c = _cs(g, rho, p)
            return (v + s * c) / (1.0 + s * v * c)

        if s * (xi - speed(rho_a, v_a, p_a)) >= 0:
            return rho_a, v_a, p_a
        rho_t, _ = self.rarefaction(a, ps, s)
        if s * (xi - speed(rho_t, vs, ps)) <= 0:
            return rho_t, vs, ps
        # inside the fan: the pressure whose characteristic speed is xi
        def G(p):
            rho, v = self.rarefaction(a, p, s)
            return s * (speed(rho, v, p) - xi)
        p = _bisect(G, ps, p_a)
        rho, v = self.rarefaction(a, p, s)
        return rho, v, p
