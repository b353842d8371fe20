"""Exact Sod shock-tube solution (TEST INFRASTRUCTURE ONLY).

Restates the reference's ``RiemannProblem:exactSolution``
(``hydro/init/euler.lua:122-245``, after the Fortran routine it cites): the
star-region pressure P3 is the root of

    f(P3) = -2 CsL (1 - (P3/PL)^((g-1)/(2g))) / (CsR (g-1))
            + (P3/PR - 1) * ((1 - mu^2) / (g (mu^2 + P3/PR)))^(1/2),

with mu^2 = (g-1)/(g+1), followed by the five-region similarity solution.  The
reference hard-codes mu^2 = 0.25 (exact only for g = 5/3); this restatement
uses mu^2 from g, which is identical for the g = 5/3 problems whose recorded
errors pin the oracle.  The reference iterates Newton with an analytic
derivative; here the same root is found with a bracketing solver.
"""
import math

import numpy as np


def sod_star_pressure(rhoL, PL, rhoR, PR, gamma):
    muSq = (gamma - 1) / (gamma + 1)
    CsL = math.sqrt(gamma * PL / rhoL)
    CsR = math.sqrt(gamma * PR / rhoR)

    def f(P3):
        return (-2 * CsL * (1 - (P3 / PL) ** ((gamma - 1) / (2 * gamma))) / (CsR * (gamma - 1))
                + (P3 / PR - 1) * ((1 - muSq) / (gamma * (muSq + P3 / PR))) ** 0.5)

    lo, hi = min(PL, PR), max(PL, PR)
    flo, fhi = f(lo), f(hi)
    assert flo * fhi <= 0, "star pressure not bracketed"
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        fm = f(mid)
        if (fm < 0) == (flo < 0):
            lo, flo = mid, fm
        else:
            hi, fhi = mid, fm
        if hi - lo <= 1e-16 * max(1.0, abs(mid)):
            break
    return 0.5 * (lo + hi)


def sod_exact(t, x, rhoL=1.0, PL=1.0, rhoR=0.125, PR=0.1, gamma=5.0 / 3.0):
    """Returns (rho, mx, my, mz, ETotal) arrays at positions x (diaphragm at 0), time t > 0."""
    x = np.asarray(x, dtype=np.float64)
    vL = vR = 0.0
    muSq = (gamma - 1) / (gamma + 1)
    CsL = math.sqrt(gamma * PL / rhoL)
    P3 = sod_star_pressure(rhoL, PL, rhoR, PR, gamma)
    P4 = P3
    rho3 = rhoL * (P3 / PL) ** (1 / gamma)
    v3 = vR + 2 * CsL / (gamma - 1) * (1 - (P3 / PL) ** ((gamma - 1) / (2 * gamma)))
    v4 = v3
    rho4 = rhoR * (P4 + muSq * PR) / (PR + muSq * P4)
    vshock = v4 * rho4 / (rho4 - rhoR)
    vtail = CsL - v4 / (1 - muSq)
    s1, s2, s3, s4 = -CsL, -vtail, v3, vshock
    xi = x / t
    rho = np.empty_like(x)
    vx = np.empty_like(x)
    P = np.empty_like(x)
    r1 = xi < s1
    r2 = (~r1) & (xi < s2)
    r3 = (~r1) & (~r2) & (xi < s3)
    r4 = (~r1) & (~r2) & (~r3) & (xi < s4)
    r5 = ~(r1 | r2 | r3 | r4)
    rho[r1], vx[r1], P[r1] = rhoL, vL, PL
    base = -muSq * (x[r2] / (CsL * t)) + (1 - muSq)
    vx[r2] = (1 - muSq) * (x[r2] / t + CsL)
    rho[r2] = rhoL * base ** (2 / (gamma - 1))
    P[r2] = PL * base ** (2 * gamma / (gamma - 1))
    rho[r3], vx[r3], P[r3] = rho3, v3, P3
    rho[r4], vx[r4], P[r4] = rho4, v4, P4
    rho[r5], vx[r5], P[r5] = rhoR, vR, PR
    EInt = P / (gamma - 1)
    EKin = 0.5 * rho * vx * vx
    z = np.zeros_like(x)
    return rho, rho * vx, z, z, EKin + EInt
