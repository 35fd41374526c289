"""The exact Riemann solver used by the shock-tube checks, pinned to the
published star state of the standard Sod problem (rho, u, p) = (1, 0, 1) |
(0.125, 0, 0.1), gamma = 1.4: p* = 0.30313, u* = 0.92745, rho*_L = 0.42632,
rho*_R = 0.26557 (five digits)."""
import numpy as np

from _riemann import sample, star_state


def test_sod_star_state():
    left, right = (1.0, 0.0, 1.0), (0.125, 0.0, 0.1)
    ps, us = star_state(left, right, 1.4)
    assert abs(ps - 0.30313) < 1e-5 and abs(us - 0.92745) < 1e-5
    s = np.array([0.5, 1.2])     # between the contact (0.927) and the shock (1.752): right star state
    r = sample(left, right, 1.4, s)
    assert abs(r[1, 0] - 0.26557) < 1e-5 and abs(r[1, 2] - 0.30313) < 1e-5
    rl = sample(left, right, 1.4, np.array([0.9]))   # left of the contact, behind the rarefaction
    assert abs(rl[0, 0] - 0.42632) < 1e-5


def test_far_states_and_symmetry():
    left, right = (1.0, 0.0, 1.0), (0.25, 0.0, 0.1795)
    r = sample(left, right, 5.0 / 3.0, np.array([-10.0, 10.0]))
    assert np.allclose(r[0], left) and np.allclose(r[1], right)
    # mirrored problem: the solution mirrors
    a = sample(left, right, 5.0 / 3.0, np.linspace(-2, 2, 41))
    b = sample(right, left, 5.0 / 3.0, -np.linspace(-2, 2, 41))
    assert np.allclose(a[:, 0], b[:, 0]) and np.allclose(a[:, 1], -b[:, 1]) and np.allclose(a[:, 2], b[:, 2])
