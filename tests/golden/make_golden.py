"""Generate the golden fixtures from the reference's own test data.

Runs only where the reference source tree is available (its root is the
first argument, or SPHERAL_REFERENCE_ROOT): it imports
tests/functional/Hydro/Sod/SodAnalyticSolution.py (a pure-Python module) for
sod_analytic.npz, and reads the Evrard collapse comparison profiles of
tests/functional/EvrardSphericalCollapse/{rho,vel,entropy}.dat for
evrard_profiles.npz.  The outputs are committed and read by the tests and
the bench.

Configuration: the 3-D planar Sod tube of spheral_gb300.problems.sod (x in
[0, 2], interface at x = 1, rho 1 / 0.25, P 1 / 0.1795, gamma 5/3), profiles
of density, velocity, specific energy and pressure at t = 0.05, 0.10, 0.15
on 401 points.
"""
import argparse
import os
import sys

import numpy as np


def _paths(root):
    """Directories of the reference's Sod and Evrard test data under the
    root of a Spheral source tree."""
    return (os.path.join(root, "tests", "functional", "Hydro", "Sod"),
            os.path.join(root, "tests", "functional", "EvrardSphericalCollapse"))


def main(root, out=os.path.join(os.path.dirname(os.path.abspath(__file__)), "sod_analytic.npz")):
    REF, EVRARD = _paths(root)
    sys.path.insert(0, REF)
    from SodAnalyticSolution import SodSolutionGasGas
    g = 5.0 / 3.0
    x = [2.0 * k / 400.0 for k in range(401)]
    data = {"x": np.array(x)}
    for t in (0.05, 0.10, 0.15):
        sol = SodSolutionGasGas(nPoints=401, gamma1=g, gamma2=g, rho1=1.0, P1=1.0, rho2=0.25, P2=0.1795,
                                x0=0.0, x1=1.0, x2=2.0, h1=0.01, h2=0.01)
        xs, v, u, rho, P, h, gam = sol.solution(t, list(x))
        key = "t%.2f" % t
        data[key + "_rho"] = np.array(rho)
        data[key + "_v"] = np.array(v)
        data[key + "_u"] = np.array(u)
        data[key + "_P"] = np.array(P)
    np.savez(out, **data)
    print("wrote", out)
    evrard(EVRARD)


def evrard(EVRARD, out=os.path.join(os.path.dirname(os.path.abspath(__file__)), "evrard_profiles.npz")):
    """Radial profiles at t = 0.8 of the Evrard collapse (columns r, value)."""
    data = {}
    for name in ("rho", "vel", "entropy"):
        a = np.loadtxt(os.path.join(EVRARD, name + ".dat"))
        data[name + "_r"] = a[:, 0]
        data[name] = a[:, 1]
    np.savez(out, **data)
    print("wrote", out)


if __name__ == "__main__":
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("reference_root", nargs="?", default=os.environ.get("SPHERAL_REFERENCE_ROOT"),
                    help="root of the Spheral source tree (default: $SPHERAL_REFERENCE_ROOT)")
    a = ap.parse_args()
    if not a.reference_root:
        ap.error("give the Spheral source root as an argument or in SPHERAL_REFERENCE_ROOT")
    main(a.reference_root)
