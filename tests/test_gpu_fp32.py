"""GPU checks of the mixed-precision mode (FP32 pair sweeps on cell-relative
positions, compensated sums, FP64 integration and energy update).

Tolerances (stated): neighbour sets exact (the FP32 pre-filter defers to the
exact FP64 criterion near the threshold); derivatives within 2e-5 normwise of
the FP64 oracle; equal-mass boxes conserve total energy to 1e-10 and momentum
to 1e-9 relative over ten steps (pair forces are bitwise antisymmetric; the
residual is the compensated-sum rounding of the per-node acceleration and of
the FP32 energy shares, versus ~1e-7 for plain FP32 sums)."""
import numpy as np
import pytest

from spheral_gb300 import problems

from _parity import compare_fields, ordered_pairs_from_oracle, periodic_axes

pytestmark = pytest.mark.gpu

CASES = {
    "periodic": lambda: problems.random_box(n_side=12, seed=21, boundaries="periodic"),
    "reflecting": lambda: problems.random_box(n_side=12, seed=22, boundaries="reflecting"),
    "kh": lambda: problems.kelvin_helmholtz(n1=16),
}
FP32_DERIVS = ["massDensitySum", "DvDt", "DepsDt", "DvDx", "gradRho", "M", "maxViscousPressure", "DHDt", "Hideal",
               "massZerothMoment"]


def _pair(oracle_mod, make):
    from spheral_gb300.engine import Engine
    p = make()
    eng = Engine.from_problem(p, precision="fp32")
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    return p, eng, orc


@pytest.mark.parametrize("case", list(CASES))
def test_fp32_neighbor_sets_exact(native_lib, oracle_mod, case):
    p, eng, orc = _pair(oracle_mod, CASES[case])
    i, j, im = eng.pairs()
    got = set(zip(i.tolist(), j.tolist(), im.tolist()))
    assert got == ordered_pairs_from_oracle(orc, periodic_axes(p))


@pytest.mark.parametrize("case", list(CASES))
def test_fp32_derivatives_close(native_lib, oracle_mod, case):
    p, eng, orc = _pair(oracle_mod, CASES[case])
    eng.evaluate_derivatives()
    orc.evaluate_derivatives()
    bad = compare_fields(eng, orc, FP32_DERIVS, 2e-5)
    assert not bad, bad


@pytest.mark.parametrize("case", list(CASES))
def test_fp32_density_and_gradh_close(native_lib, oracle_mod, case):
    p, eng, orc = _pair(oracle_mod, CASES[case])
    bad = compare_fields(eng, orc, ["omegaGradh"], 2e-6)
    assert not bad, bad
    eng.sum_density()
    orc.sum_density()
    bad = compare_fields(eng, orc, ["massDensity"], 2e-6)
    assert not bad, bad


def test_fp32_conserves_momentum_and_energy(native_lib):
    from spheral_gb300.engine import Engine
    p = problems.turbulent_box(n_side=16, seed=7)
    eng = Engine.from_problem(p, precision="fp32")
    eng.initialize()
    c0 = eng.conservation()
    eng.advance(10)
    c1 = eng.conservation()
    scale = np.sum(p.mass * np.linalg.norm(p.vel, axis=1))
    assert abs(c1[7] - c0[7]) <= 1e-10 * abs(c0[7]), (c1[7] - c0[7]) / c0[7]
    assert np.all(np.abs(c1[1:4] - c0[1:4]) <= 1e-9 * scale), (c1[1:4] - c0[1:4]) / scale


def test_fp32_tracks_fp64(native_lib):
    from spheral_gb300.engine import Engine
    p = problems.kelvin_helmholtz(n1=16)
    a = Engine.from_problem(p, precision="fp32")
    b = Engine.from_problem(p, precision="fp64")
    for e in (a, b):
        e.initialize()
        e.advance(5)
    for name, tol in (("position", 1e-6), ("velocity", 1e-4), ("specificThermalEnergy", 1e-5),
                      ("massDensity", 1e-5)):
        x, y = a.field(name), b.field(name)
        err = np.max(np.abs(x - y)) / np.max(np.abs(y))
        assert err < tol, (name, err)


@pytest.mark.parametrize("case", list(CASES))
def test_fp32_step_dt_close(native_lib, oracle_mod, case):
    """The time step of the mixed step (density sum and dt vote fused, node
    limits in FP32) within 1e-5 of the FP64 oracle's over three steps."""
    p, eng, orc = _pair(oracle_mod, CASES[case])
    for _ in range(3):
        dg = eng.step()
        do = orc.step()
        assert abs(dg - do) <= 1e-5 * do, (dg, do)


@pytest.mark.parametrize("case", ["periodic", "kh"])
def test_fp32_plain_sums_close(native_lib, oracle_mod, case):
    # the FP32-relative mode of the throughput sweep (SPHGPU_PRECISION_FP32_PLAIN):
    # the same FP32 sweeps with plain sums, same neighbour sets, derivatives
    # within the mixed mode's 2e-5 of the FP64 oracle
    from spheral_gb300.engine import Engine
    p = CASES[case]()
    eng = Engine.from_problem(p, precision="fp32_plain")
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    i, j, im = eng.pairs()
    assert set(zip(i.tolist(), j.tolist(), im.tolist())) == ordered_pairs_from_oracle(orc, periodic_axes(p))
    eng.evaluate_derivatives()
    orc.evaluate_derivatives()
    bad = compare_fields(eng, orc, FP32_DERIVS, 2e-5)
    assert not bad, bad
    eng.advance(3)
