"""NBSplineKernel (src/Kernel/NBSplineKernel.cc) in the oracle and its
TableKernel:

* order 3 is the cubic B-spline: its Simpson-normalised values equal the
  analytic BSplineKernel (normalisation 1/pi) to 1e-10;
* every odd order integrates to one over 3-D space (Gauss-Legendre on the
  knot intervals, exact for the polynomial pieces, 1e-9), vanishes at its extent (order + 1) / 2 and has
  W' = dW/deta (finite differences); even orders keep the reference's
  integer-division extent, which cuts the spline short of its support
  (order 2: extent 1 of 1.5), so they are truncated where the table ends;
* the table reproduces the analytic kernel far inside the reference's own
  table tolerances (tests/unit/Kernel/testTableKernel.py: W 1e-3, grad W 1e-2).
"""
import numpy as np
import pytest
from scipy import integrate

from spheral_gb300 import problems


def _bspline(eta):
    eta = np.asarray(eta, dtype=float)
    w = np.where(eta < 1.0, 1.0 - 1.5 * eta ** 2 + 0.75 * eta ** 3, np.where(eta < 2.0, 0.25 * (2.0 - eta) ** 3, 0.0))
    return w / np.pi


def test_order3_is_the_cubic_bspline(oracle_mod):
    eta = np.linspace(0.0, 2.2, 111)
    got = np.array([oracle_mod.nbspline_value(3, e) for e in eta])
    assert np.abs(got - _bspline(eta)).max() < 1e-10


@pytest.mark.parametrize("order", [3, 5, 7, 9])
def test_normalised_and_consistent(oracle_mod, order):
    ext = float((order + 1) // 2)
    # Gauss-Legendre on the spline's unit knot intervals: r^2 W is a
    # polynomial of degree order + 2 <= 11 on each, which 8 nodes integrate exactly
    xg, wg = np.polynomial.legendre.leggauss(8)
    val = 0.0
    for a in np.arange(0.0, ext):
        r = a + 0.5 * (xg + 1.0)
        val += 0.5 * sum(w * 4 * np.pi * x * x * oracle_mod.nbspline_value(order, x) for x, w in zip(r, wg))
    assert abs(val - 1.0) < 1e-9
    assert oracle_mod.nbspline_value(order, ext) == 0.0
    for e in np.linspace(0.05, ext - 0.05, 13):
        d = 1e-6
        fd = (oracle_mod.nbspline_value(order, e + d) - oracle_mod.nbspline_value(order, e - d)) / (2 * d)
        assert abs(fd - oracle_mod.nbspline_grad(order, e)) < 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("order", [3, 5])
def test_table_matches_analytic(oracle_mod, order):
    p = problems.random_box(n_side=12)
    p.config.update(kernel="nbspline", kernel_order=order)
    o = oracle_mod.Oracle(p)
    ext = float((order + 1) // 2)
    for e in np.linspace(0.0, ext * 0.999, 200):
        w, g = oracle_mod.nbspline_value(order, e), oracle_mod.nbspline_grad(order, e)
        assert abs(o.kernel_value(e) - w) < 1e-6 * max(1.0, abs(w))
        assert abs(o.grad_value(e) - g) < 1e-5 * max(1.0, abs(g))


@pytest.mark.parametrize("order", [2, 4])
def test_even_orders_truncated_at_the_integer_extent(oracle_mod, order):
    ext = (order + 1) // 2
    assert oracle_mod.nbspline_value(order, ext - 1e-9) > 1e-4
    assert oracle_mod.nbspline_value(order, float(ext)) == 0.0


@pytest.mark.parametrize("kernel", ["wendland_c2", "wendland_c4"])
def test_wendland_tables_normalised(oracle_mod, kernel):
    # WendlandC2 / C4 (3-D forms, extent 1): the tabulated kernel integrates
    # to one and vanishes at the extent
    p = problems.random_box(n_side=12)
    p.config.update(kernel=kernel)
    o = oracle_mod.Oracle(p)
    val, _ = integrate.quad(lambda r: 4 * np.pi * r * r * o.kernel_value(r), 0.0, 1.0, limit=400)
    assert abs(val - 1.0) < 1e-6
    assert o.kernel_value(1.0) == 0.0 and o.kernel_value(0.0) > 0.0
