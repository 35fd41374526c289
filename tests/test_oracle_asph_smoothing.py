"""CPU checks of the oracle's ASPHSmoothingScale restatement in its
fixShape and radialOnly forms (src/SmoothingScale/ASPHSmoothingScale.cc:157-380,
IncrementASPHHtensor.cc:37-100): the tensor H is integrated with DH/Dt at
both updates of the step (fixShape: by the cube root of the determinant
ratio only) and reset at the end of the step from the zeroth moment of the
new state.

* fixShape keeps the normalised shape H / det(H)^(1/3) of every node
  through the step (limits not active).
* The end-of-step size follows the IdealH target: on a jittered lattice
  started with h 30% too large, the effective nodes per smoothing scale
  from the zeroth moment move toward nPerh.
* radialOnly: for nodes whose H has the radial direction as an eigenvector
  and no motion, it stays an eigenvector (only the radial and transverse
  scales change).
* Compatible-energy steps in either form conserve energy and momentum to
  rounding (the pair force is unchanged by the H scheme).
"""
import numpy as np
import pytest

from spheral_gb300 import problems


def _sym(a6):
    return np.array([[a6[0], a6[1], a6[2]], [a6[1], a6[3], a6[4]], [a6[2], a6[4], a6[5]]])


def _shape(h6):
    m = _sym(h6)
    return m / np.cbrt(np.linalg.det(m))


def _asph(p, **kw):
    p.config.update(smoothing_scale="asph", **kw)
    return p


def test_fixshape_keeps_the_shape(oracle_mod):
    p = _asph(problems.stretched_box(nx=14, ny=11, nz=9, seed=3), fix_shape=True)
    p.nodelists[0]["hminratio"] = 1e-3
    o = oracle_mod.Oracle(p)
    o.initialize()
    H0 = o.field("H").copy()
    for _ in range(3):
        o.step()
    H1 = o.field("H")
    err = max(np.max(np.abs(_shape(a) - _shape(b))) for a, b in zip(H0, H1))
    assert err < 1e-12
    assert np.max(np.abs(H1 - H0)) > 1e-6 * np.max(np.abs(H0))   # the size did change


def test_ideal_h_moves_toward_nperh(oracle_mod):
    p = _asph(problems.stretched_box(nx=12, ny=12, nz=12, seed=4, tilt=0.0), fix_shape=True)
    p.H = p.H / 1.3                       # h 30% too large
    o = oracle_mod.Oracle(p)
    o.initialize()
    nperh = p.nodelists[0]["nPerh"]

    def spread():
        m0 = o.field("massZerothMoment")
        return np.median(np.abs(np.array([o.nperh_lookup(v) for v in m0]) - nperh))

    o.step()
    first = spread()
    for _ in range(4):
        o.step()
    assert spread() < 0.5 * first


def test_radial_only_keeps_radial_eigenvectors_of_static_nodes(oracle_mod):
    p = _asph(problems.stretched_box(nx=10, ny=10, nz=10, seed=5, tilt=0.0, vel_scale=0.0), radial_only=True)
    p.pos = p.pos - 0.5                   # about the origin
    p.boundaries = []
    p.vel[:] = 0.0
    # H with the radial direction as an eigenvector at every node
    n = p.n
    H = np.zeros((n, 6))
    for k in range(n):
        r = p.pos[k] / np.linalg.norm(p.pos[k])
        a, b = 1.0 / 0.1, 1.0 / 0.13
        m = b * np.eye(3) + (a - b) * np.outer(r, r)
        H[k] = [m[0, 0], m[0, 1], m[0, 2], m[1, 1], m[1, 2], m[2, 2]]
    p.H = H
    o = oracle_mod.Oracle(p)
    o.initialize()
    o.step()
    H1 = o.field("H")
    x1 = o.field("position")
    worst = 0.0
    for k in range(n):
        r = x1[k] / np.linalg.norm(x1[k])
        m = _sym(H1[k])
        v = m @ r
        worst = max(worst, np.linalg.norm(v - (r @ v) * r) / np.linalg.norm(v))
    assert worst < 1e-10


@pytest.mark.parametrize("kw", [dict(fix_shape=True), dict(radial_only=True)])
def test_compatible_energy_conserved(oracle_mod, kw):
    p = _asph(problems.stretched_box(nx=10, ny=9, nz=8, seed=6), **kw)
    o = oracle_mod.Oracle(p)
    o.initialize()
    c0 = o.conservation()
    for _ in range(3):
        o.step()
    c1 = o.conservation()
    assert abs(c1[7] - c0[7]) <= 1e-12 * abs(c0[7])
    assert np.max(np.abs(c1[1:4] - c0[1:4])) <= 1e-13 * np.sum(p.mass * np.linalg.norm(p.vel, axis=1))
