"""CPU checks of the oracle's ASPHClassicSmoothingScale restatement
(src/SmoothingScale/ASPHClassicSmoothingScale.cc, SmoothingScaleUtilities.hh).

* The symmetric eigen-decomposition (the reference calls Eigen's
  SelfAdjointEigenSolver from GeomSymmetricTensor::eigenVectors) agrees with
  LAPACK on random, diagonal and degenerate tensors.
* The tensor DH/Dt reduces to -a sym(DvDx) for isotropic H = a I (no change
  under a pure rotation) and to -alpha H under a uniform expansion
  DvDx = alpha I, for any H.
* On a perfect cubic lattice the second moment is isotropic, so Hideal stays
  isotropic; on a stretched lattice its eigenvalues order like the inverse
  spacings.
* fixShape scales H without changing its shape.
* Compatible-energy steps with the ASPH H evolution conserve energy and
  momentum to rounding.
* HUpdate: IntegrateH increments H by dt DHDt at the full update, FixedH
  leaves it unchanged (SmoothingScaleBase.cc:53-82).
* radialOnly (radialEvolution): the identity for s = 1 and an unchanged
  radius; for isotropic H the radial eigenvalue scales by 1/s and the
  transverse ones by r0/r1.
"""
import numpy as np
import pytest

from spheral_gb300 import problems


def sym(a6):
    return np.array([[a6[0], a6[1], a6[2]], [a6[1], a6[3], a6[4]], [a6[2], a6[4], a6[5]]])


def six(m):
    return [m[0, 0], m[0, 1], m[0, 2], m[1, 1], m[1, 2], m[2, 2]]


def test_sym_eigen_matches_lapack(oracle_mod):
    rng = np.random.default_rng(5)
    cases = []
    for _ in range(40):
        a = rng.normal(size=(3, 3))
        cases.append(a + a.T)
    cases.append(np.diag([3.0, 1.0, 2.0]))
    cases.append(np.eye(3) * 7.0)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    cases.append(q @ np.diag([2.0, 2.0, 5.0]) @ q.T)            # a double eigenvalue
    cases.append(q @ np.diag([1e-3, 1.0, 1e3]) @ q.T)           # wide spread
    for A in cases:
        vals, vecs = oracle_mod.sym_eigen(six(A))
        assert np.allclose(np.sort(vals), np.linalg.eigvalsh(A), rtol=1e-13, atol=1e-13 * np.abs(A).max())
        assert np.allclose(vecs.T @ vecs, np.eye(3), atol=1e-13)
        assert np.allclose(vecs @ np.diag(vals) @ vecs.T, A, atol=1e-13 * np.abs(A).max())


def test_tensor_dhdt_isotropic_and_expansion(oracle_mod):
    rng = np.random.default_rng(6)
    for _ in range(10):
        a = rng.uniform(5.0, 20.0)
        D = rng.normal(size=(3, 3))
        got = sym(oracle_mod.smoothing_scale_derivative(six(a * np.eye(3)), D.ravel()))
        assert np.allclose(got, -a * 0.5 * (D + D.T), rtol=1e-12, atol=1e-12 * a)
        W = D - D.T                                                  # a pure rotation leaves isotropic H alone
        assert np.abs(oracle_mod.smoothing_scale_derivative(six(a * np.eye(3)), W.ravel())).max() < 1e-12 * a
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        H = q @ np.diag(rng.uniform(5.0, 20.0, 3)) @ q.T
        alpha = rng.normal()
        got = sym(oracle_mod.smoothing_scale_derivative(six(H), (alpha * np.eye(3)).ravel()))
        assert np.allclose(got, -alpha * H, rtol=1e-12, atol=1e-12 * np.abs(H).max())


def _hideal_eigs(o):
    return np.array([np.linalg.eigvalsh(sym(h)) for h in o.field("Hideal")])


def test_cubic_lattice_keeps_h_isotropic(oracle_mod):
    p = problems.stretched_box(nx=16, ny=16, nz=16, jitter=0.0, vel_scale=0.0, tilt=0.0, seed=3)
    p.H[:] = [1.0 / (1.51 / 16), 0.0, 0.0, 1.0 / (1.51 / 16), 0.0, 1.0 / (1.51 / 16)]
    o = oracle_mod.Oracle(p)
    o.initialize()
    o.evaluate_derivatives()
    ev = _hideal_eigs(o)
    assert np.abs(ev[:, 2] - ev[:, 0]).max() < 1e-10 * ev.max()
    # the size follows the SPH IdealH: nPerh of the lattice is already right
    assert np.allclose(ev, 16 / 1.51, rtol=2e-2)


def test_stretched_lattice_orders_hideal(oracle_mod):
    p = problems.stretched_box(nx=24, ny=18, nz=14, jitter=0.0, vel_scale=0.0, tilt=0.0, seed=4)
    o = oracle_mod.Oracle(p)
    o.initialize()
    o.evaluate_derivatives()
    hid = o.field("Hideal")
    # the principal axes stay the lattice axes; finer spacing -> larger 1/h
    assert np.abs(hid[:, [1, 2, 4]]).max() < 1e-8 * hid[:, 0].max()
    assert np.all(hid[:, 0] > hid[:, 3]) and np.all(hid[:, 3] > hid[:, 5])
    m2 = o.field("massSecondMoment")
    assert np.all(m2[:, 0] > 0) and np.all(m2[:, 3] > 0) and np.all(m2[:, 5] > 0)


def test_fix_shape_scales_h(oracle_mod):
    p = problems.stretched_box(fix_shape=True, seed=8)
    o = oracle_mod.Oracle(p)
    o.initialize()
    o.evaluate_derivatives()
    H = o.field("H")
    hid = o.field("Hideal")
    # Hideal = H / f with a per-node scalar f (limits inactive here)
    f = hid[:, 0] / H[:, 0]
    assert np.allclose(hid, H * f[:, None], rtol=1e-10, atol=1e-10 * np.abs(hid).max())


@pytest.mark.parametrize("boundaries", ["periodic", "reflecting"])
def test_asph_steps_conserve(oracle_mod, boundaries):
    p = problems.stretched_box(boundaries=boundaries, seed=9)
    o = oracle_mod.Oracle(p)
    o.initialize()
    c0 = o.conservation()
    for _ in range(4):
        o.step()
    c1 = o.conservation()
    assert abs(c1[7] - c0[7]) < 1e-12 * abs(c0[7])
    if boundaries == "periodic":
        assert np.abs(c1[1:4] - c0[1:4]).max() < 1e-12 * np.sqrt(2.0 * c0[0] * c0[4])
    H = o.field("H")
    ev = np.array([np.linalg.eigvalsh(sym(h)) for h in H])
    assert np.all(ev > 0.0)
    assert np.abs(H[:, [1, 2, 4]]).max() > 0.0       # the tensor evolves with off-diagonal terms


@pytest.mark.parametrize("h_update", ["integrate", "fixed"])
def test_h_update_options(oracle_mod, h_update):
    # IntegrateH: the full update increments H by dt DHDt from the midpoint
    # derivatives (IncrementBoundedState); FixedH: H never changes
    p = problems.stretched_box(seed=10)
    p.config["h_update"] = h_update
    o = oracle_mod.Oracle(p)
    o.initialize()
    H0 = o.field("H")
    c0 = o.conservation()
    dt = o.step()
    H1 = o.field("H")
    if h_update == "fixed":
        assert np.array_equal(H1, H0)
    else:
        want = H0 + dt * o.field("DHDt")
        assert np.allclose(H1, want, rtol=1e-12, atol=1e-12 * np.abs(H0).max())
    assert abs(o.conservation()[7] - c0[7]) < 1e-12 * abs(c0[7])


def test_radial_evolution(oracle_mod):
    rng = np.random.default_rng(12)
    for _ in range(5):
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        H = q @ np.diag(rng.uniform(5.0, 20.0, 3)) @ q.T
        x = rng.normal(size=3)
        got = sym(oracle_mod.radial_evolution(six(H), x, 1.0, np.linalg.norm(x)))
        assert np.allclose(got, H, rtol=1e-12, atol=1e-12 * np.abs(H).max())
        a, s, fr = 10.0, 1.3, 1.1
        got = sym(oracle_mod.radial_evolution(six(a * np.eye(3)), x, s, np.linalg.norm(x) / fr))
        nh = x / np.linalg.norm(x)
        assert abs(nh @ got @ nh - a / s) < 1e-12 * a
        t = np.cross(nh, [0.3, -0.2, 0.9])
        t /= np.linalg.norm(t)
        assert abs(t @ got @ t - a / fr) < 1e-12 * a


def test_radial_only_steps_conserve(oracle_mod):
    p = problems.stretched_box(seed=11)
    p.config["radial_only"] = True
    o = oracle_mod.Oracle(p)
    o.initialize()
    c0 = o.conservation()
    for _ in range(3):
        o.step()
    assert abs(o.conservation()[7] - c0[7]) < 1e-12 * abs(c0[7])
