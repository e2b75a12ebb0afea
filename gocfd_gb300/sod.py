"""Exact Sod shock-tube solution, for the shock-tube post-processing
(the reference compares its shocktube runs with it, euler.go:222-250).

Restates model_problems/Euler1D/sod_shock_tube/analytic_sod.go: NewSOD/calc
(:22-61) for the wave positions x1..x4 and the post-shock state, Getx (:63-103)
for the piecewise solution, fzero/sod_func (:131-162) for the post-shock
pressure (a secant iteration on the pressure equation, started at pi), and
Get (:105-129) for the reference's sample abscissae.  Left state (1, 1, 0),
right state (0.125, 0.1, 0), gamma = 1.4, diaphragm at x0 = 0.5 on [0, 1].
Pinned by TestSOD's golden vectors (analytic_sod_test.go:16-30).
"""
import math

import numpy as np

GAMMA = 1.4
LEFT = (1.0, 1.0, 0.0)    # rho, p, u
RIGHT = (0.125, 0.1, 0.0)


def _c(rho, p, g=GAMMA):
    return math.sqrt(g * p / rho)


def _sod_func(P, g=GAMMA):
    rho_l, P_l = LEFT[0], LEFT[1]
    rho_r, P_r = RIGHT[0], RIGHT[1]
    mu2 = (g - 1) / (g + 1)
    return ((P - P_r) * math.sqrt((1 - mu2) / (rho_r * (P + mu2 * P_r)))
            - (P_l ** ((g - 1) / (2 * g)) - P ** ((g - 1) / (2 * g)))
            * math.sqrt(((1 - mu2 * mu2) * P_l ** (1 / g)) / (mu2 * mu2 * rho_l)))


def _fzero(f, start, tol=1e-7):
    start_old = start / 2
    res = f(start_old)
    while abs(res) > tol:
        res_new = f(start)
        deriv = (start - start_old) / (res_new - res)
        start_new = abs(start - res_new * deriv)
        start_old, start, res = start, start_new, res_new
    return start


class SodExact:
    def __init__(self, t, g=GAMMA, x_min=0.0, x_max=1.0):
        self.g, self.t, self.x_min, self.x_max = g, t, x_min, x_max
        mu2 = (g - 1) / (g + 1)
        rl, pl, ul = LEFT
        rr, pr, ur = RIGHT
        P_post = _fzero(_sod_func, math.pi)
        self.rho_middle = rl * (P_post / pl) ** (1.0 / g)
        self.x0 = 0.5 * (x_max + x_min)
        rho_post = rr * ((P_post / pr) + mu2) / (1 + mu2 * (P_post / pr))
        u_post = ur + (P_post - pr) / math.sqrt(0.5 * rr * ((g + 1) * P_post + (g - 1) * pr))
        self.post = (rho_post, P_post, u_post)
        v_shock = u_post * (rho_post / rr) / ((rho_post / rr) - 1.0)
        cl = _c(rl, pl, g)
        self.x1 = self.x0 - cl * t
        self.x3 = self.x0 + u_post * t
        self.x4 = self.x0 + v_shock * t
        c2 = cl - 0.5 * (g - 1.0) * u_post
        self.x2 = self.x0 + t * (u_post - c2)

    def getx(self, x):
        """(rho, p, u, E, rho u) at x."""
        g = self.g
        mu2 = (g - 1) / (g + 1)
        rl, pl, ul = LEFT
        rr, pr, ur = RIGHT
        cl = _c(rl, pl, g)
        if x < self.x1:
            rho, p, u = rl, pl, ul
        elif x <= self.x2:
            c = mu2 * ((self.x0 - x) / self.t) + (1.0 - mu2) * cl
            rho = rl * (c / cl) ** (2 / (g - 1))
            p = pl * (rho / rl) ** g
            u = (1.0 - mu2) * ((-(self.x0 - x) / self.t) + cl)
        elif x <= self.x3:
            rho, p, u = self.rho_middle, self.post[1], self.post[2]
        elif x <= self.x4:
            rho, p, u = self.post
        else:
            rho, p, u = rr, pr, ur
        E = p / (g - 1.0) + 0.5 * u * u * rho
        return rho, p, u, E, rho * u

    def density(self, x):
        return np.array([self.getx(float(v))[0] for v in np.ravel(x)]).reshape(np.shape(x))

    def sample(self):
        """The reference's Get(): abscissae around the wave positions and density there."""
        tol = 1e-4
        mid = (self.x2 - self.x1) / 10.0
        X = [self.x_min, self.x1 - tol, self.x1 + tol] + [self.x1 + i * mid for i in range(1, 10)] + \
            [self.x1 + 10 * mid - 2 * tol, self.x2 - tol, self.x2 + tol, self.x3 - tol, self.x3 + tol,
             self.x4 - tol, self.x4 + tol, self.x_max]
        return np.array(X), np.array([self.getx(x)[0] for x in X])
