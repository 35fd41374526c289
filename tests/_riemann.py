"""Exact solution of the 1-D Riemann problem for an ideal gas (test
infrastructure: the analytic reference of the shock-tube checks).

The star-region pressure solves f_L(p) + f_R(p) + (u_R - u_L) = 0 with the
shock / rarefaction branches of each side (the classic exact Riemann solver
of gas dynamics); the solution is then sampled on the similarity variable
x / t.  States are (rho, u, p)."""
import numpy as np


def _f(p, rho, pk, gamma):
    """f_K(p) and its derivative for one side of the interface."""
    a = np.sqrt(gamma * pk / rho)
    if p > pk:   # shock
        A = 2.0 / ((gamma + 1.0) * rho)
        B = (gamma - 1.0) / (gamma + 1.0) * pk
        q = np.sqrt(A / (p + B))
        return (p - pk) * q, q * (1.0 - 0.5 * (p - pk) / (p + B))
    e = (gamma - 1.0) / (2.0 * gamma)   # rarefaction
    return 2.0 * a / (gamma - 1.0) * ((p / pk) ** e - 1.0), (p / pk) ** (-(gamma + 1.0) / (2.0 * gamma)) / (rho * a)


def star_state(left, right, gamma):
    rl, ul, pl = left
    rr, ur, pr = right
    p = 0.5 * (pl + pr)
    for _ in range(100):
        fl, dl = _f(p, rl, pl, gamma)
        fr, dr = _f(p, rr, pr, gamma)
        dp = (fl + fr + ur - ul) / (dl + dr)
        p = max(1e-12, p - dp)
        if abs(dp) < 1e-14 * p:
            break
    fl, _ = _f(p, rl, pl, gamma)
    fr, _ = _f(p, rr, pr, gamma)
    return p, 0.5 * (ul + ur) + 0.5 * (fr - fl)


def sample(left, right, gamma, s):
    """(rho, u, p) at the similarity coordinates s = (x - x0) / t."""
    rl, ul, pl = left
    rr, ur, pr = right
    ps, us = star_state(left, right, gamma)
    gm, gp = gamma - 1.0, gamma + 1.0
    out = np.zeros((len(s), 3))
    al, ar = np.sqrt(gamma * pl / rl), np.sqrt(gamma * pr / rr)
    for k, x in enumerate(s):
        if x <= us:   # left of the contact
            if ps > pl:   # left shock
                sl = ul - al * np.sqrt(gp / (2 * gamma) * ps / pl + gm / (2 * gamma))
                if x < sl:
                    out[k] = (rl, ul, pl)
                else:
                    out[k] = (rl * (ps / pl + gm / gp) / (gm / gp * ps / pl + 1.0), us, ps)
            else:   # left rarefaction
                als = al * (ps / pl) ** (gm / (2 * gamma))
                if x < ul - al:
                    out[k] = (rl, ul, pl)
                elif x > us - als:
                    out[k] = (rl * (ps / pl) ** (1.0 / gamma), us, ps)
                else:
                    u = 2.0 / gp * (al + gm / 2 * ul + x)
                    c = 2.0 / gp * (al + gm / 2 * (ul - x))
                    r = rl * (c / al) ** (2.0 / gm)
                    out[k] = (r, u, pl * (c / al) ** (2 * gamma / gm))
        else:   # right of the contact
            if ps > pr:   # right shock
                sr = ur + ar * np.sqrt(gp / (2 * gamma) * ps / pr + gm / (2 * gamma))
                if x > sr:
                    out[k] = (rr, ur, pr)
                else:
                    out[k] = (rr * (ps / pr + gm / gp) / (gm / gp * ps / pr + 1.0), us, ps)
            else:   # right rarefaction
                ars = ar * (ps / pr) ** (gm / (2 * gamma))
                if x > ur + ar:
                    out[k] = (rr, ur, pr)
                elif x < us + ars:
                    out[k] = (rr * (ps / pr) ** (1.0 / gamma), us, ps)
                else:
                    u = 2.0 / gp * (-ar + gm / 2 * ur + x)
                    c = 2.0 / gp * (ar - gm / 2 * (ur - x))
                    r = rr * (c / ar) ** (2.0 / gm)
                    out[k] = (r, u, pr * (c / ar) ** (2 * gamma / gm))
    return out
