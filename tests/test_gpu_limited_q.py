"""LimitedMonaghanGingoldViscosity (the SPH() factory default Q) on the GPU
against the oracle's restatement of LimitedMonaghanGingoldViscosity::QPiij and
of ArtificialViscosityHandle's DvDx copy at every postStateUpdate.

Tolerances: FP64 — one step <= 1e-11 and five steps <= 1e-9 normwise (the
limiter's ratio and exp are smooth, so only summation order differs);
mixed — derivatives after three steps within 5e-5 normwise of the FP64 oracle,
energy conserved to 1e-10 over five steps (the limited pair force stays
bitwise antisymmetric)."""
import numpy as np
import pytest

from spheral_gb300 import problems

from _parity import STATE_FIELDS, compare_fields

pytestmark = pytest.mark.gpu


def _limited(p):
    p.config["viscosity"] = "limited_monaghan_gingold"
    return p


CASES = {
    "periodic": lambda: _limited(problems.random_box(n_side=12, seed=61, boundaries="periodic")),
    "reflecting": lambda: _limited(problems.random_box(n_side=12, seed=62, boundaries="reflecting")),
    "two_lists": lambda: _limited(problems.random_box(n_side=12, seed=63, boundaries="periodic", two_lists=True)),
    "sod": lambda: _limited(problems.sod(nx1=16, ny1=20)),
}


def _pair(oracle_mod, make, precision="fp64"):
    from spheral_gb300.engine import Engine
    p = make()
    eng = Engine.from_problem(p, precision=precision)
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    return p, eng, orc


@pytest.mark.parametrize("case", list(CASES))
def test_limited_q_step_parity(native_lib, oracle_mod, case):
    p, eng, orc = _pair(oracle_mod, CASES[case])
    dg, do = eng.step(), orc.step()
    assert abs(dg - do) <= 1e-12 * do
    bad = compare_fields(eng, orc, STATE_FIELDS, 1e-11)
    assert not bad, bad
    for _ in range(4):
        eng.step()
        orc.step()
    bad = compare_fields(eng, orc, STATE_FIELDS + ["DvDt", "DepsDt", "DvDx", "maxViscousPressure",
                                                   "ArtificialViscosityVelocityGradient"], 1e-9)
    assert not bad, bad


@pytest.mark.parametrize("case", ["periodic", "reflecting"])
def test_limited_q_mixed_close(native_lib, oracle_mod, case):
    p, eng, orc = _pair(oracle_mod, CASES[case], precision="fp32")
    for _ in range(3):
        eng.step()
        orc.step()
    bad = compare_fields(eng, orc, ["position", "velocity", "specificThermalEnergy", "DvDt", "DepsDt",
                                    "maxViscousPressure"], 5e-5)
    assert not bad, bad


def test_limited_q_mixed_conserves_energy(native_lib):
    from spheral_gb300.engine import Engine
    p = _limited(problems.turbulent_box(16, 9))
    eng = Engine.from_problem(p, precision="fp32")
    eng.initialize()
    c0 = eng.conservation()
    eng.advance(5)
    c1 = eng.conservation()
    assert abs(c1[7] - c0[7]) <= 1e-10 * abs(c0[7])
