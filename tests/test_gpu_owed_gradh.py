"""The end-of-step grad-h correction (postStateUpdate of
src/SPH/SPHHydroBase.cc, computed after the full update of
src/Integrator/CheapSynchronousRK2.cc:109-113) is owed by the GPU step: the
next step recomputes it at its half-step postStateUpdate before anything reads
it, so it is evaluated only when the state is read from outside a step.  Each
read settles it with the values an eager evaluation gives.

Every entry that reads the state straight after a step is checked against the
oracle (which evaluates it eagerly): the field itself, a derivative
evaluation, a density sum, the dt vote, and a checkpoint restored into a fresh
engine.  Cases: FP64 with open boundaries (owed) and reflecting walls (the
FP64 sweep would see positions the walls moved, so it stays eager there), the
mixed mode with periodic and reflecting boundaries (owed: its sweep reads the
FP32 mirror the update wrote).

Tolerances: FP64 1e-9 after three steps (as the step parity tests); mixed mode
5e-5 of the FP64 oracle."""
import numpy as np
import pytest

from spheral_gb300 import problems

from _parity import DERIV_FIELDS, compare_fields

pytestmark = pytest.mark.gpu

CASES = [("fp64", "open"), ("fp64", "reflecting"), ("fp32", "periodic"), ("fp32", "reflecting")]


def _stepped(oracle_mod, precision, boundaries, nsteps=3):
    from spheral_gb300.engine import Engine
    p = problems.random_box(n_side=10, seed=131, boundaries=boundaries, vel_scale=0.2)
    eng = Engine.from_problem(p, precision=precision)
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    for _ in range(nsteps):
        eng.step()
        orc.step()
    return p, eng, orc


def _tol(precision):
    return 1e-9 if precision == "fp64" else 5e-5


@pytest.mark.parametrize("precision,boundaries", CASES)
def test_owed_omega_field(native_lib, oracle_mod, precision, boundaries):
    p, eng, orc = _stepped(oracle_mod, precision, boundaries)
    bad = compare_fields(eng, orc, ["omegaGradh", "massDensity", "H"], _tol(precision))
    assert not bad, bad
    om = eng.field("omegaGradh")
    assert np.all(np.isfinite(om)) and np.abs(om - 1.0).max() > 1e-4   # really corrected


@pytest.mark.parametrize("precision,boundaries", CASES)
def test_owed_omega_derivatives(native_lib, oracle_mod, precision, boundaries):
    p, eng, orc = _stepped(oracle_mod, precision, boundaries)
    eng.evaluate_derivatives()          # the first read after the step
    orc.evaluate_derivatives()
    tol = 1e-9 if precision == "fp64" else 1e-4
    bad = compare_fields(eng, orc, ["DvDt", "DepsDt", "DvDx", "DHDt", "omegaGradh"], tol)
    assert not bad, bad


@pytest.mark.parametrize("precision,boundaries", CASES)
def test_owed_omega_density_and_dt(native_lib, oracle_mod, precision, boundaries):
    p, eng, orc = _stepped(oracle_mod, precision, boundaries)
    dg, _ = eng.dt()
    do = orc.hydro_dt()
    assert abs(dg - do) <= (1e-10 if precision == "fp64" else 1e-5) * do
    eng.sum_density()
    orc.sum_density()
    bad = compare_fields(eng, orc, ["massDensity", "omegaGradh"], _tol(precision))
    assert not bad, bad


@pytest.mark.parametrize("precision,boundaries", CASES)
def test_owed_omega_checkpoint(native_lib, oracle_mod, precision, boundaries):
    from spheral_gb300.engine import Engine
    p, eng, orc = _stepped(oracle_mod, precision, boundaries)
    image = eng.checkpoint()
    again = Engine(p.config, precision=precision)
    for k, nl in enumerate(p.nodelists):
        again.set_nodelist(k, nl["nPerh"], nl["hmin"], nl["hmax"], nl["rhoMin"], nl["rhoMax"], nl["gamma"])
    for b in p.boundaries:
        again.add_boundary(b["type"], b["axis"], b["lo"], b["hi"], b.get("wall_high", 0))
    again.restore(image)
    assert np.array_equal(again.field("omegaGradh"), eng.field("omegaGradh"))
    bad = compare_fields(again, orc, ["omegaGradh"], _tol(precision))
    assert not bad, bad
    # the restored run and the original continue identically
    eng.step()
    again.step()
    assert np.array_equal(again.field("position"), eng.field("position"))
    assert np.array_equal(again.field("omegaGradh"), eng.field("omegaGradh"))
