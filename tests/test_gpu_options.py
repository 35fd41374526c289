"""The SPH() package options on the GPU against the oracle: each option of
the reference factory (src/SPH/SPHHydros.py:9-33) and of the MG Q switched
on its own, plus the factory's own defaults (XSPH on, the limited Q).

Tolerances as in test_gpu_parity: FP64 derivatives <= 1e-12 after one
evaluation, one step <= 1e-11, four more steps <= 1e-9; mixed mode
derivatives within 5e-5 of the FP64 oracle."""
import pytest

from spheral_gb300 import problems

from _parity import DERIV_FIELDS, STATE_FIELDS, compare_fields

pytestmark = pytest.mark.gpu

OPTIONS = {
    "xsph": dict(xsph=True),
    "integrate_density": dict(density_update=1),
    "tensile": dict(eps_tensile=0.3, n_tensile=4.0),
    "linear_in_expansion": dict(linear_in_expansion=True),
    "quadratic_in_expansion": dict(quadratic_in_expansion=True),
    "no_compatible_energy": dict(compatible_energy=False),
    "no_gradh": dict(gradh_correction=False),
    "no_velocity_gradient_correction": dict(correct_velocity_gradient=False),
    "velocity_magnitude_dt": dict(use_velocity_magnitude_for_dt=True),
    "sph_factory_defaults": dict(xsph=True, viscosity="limited_monaghan_gingold"),
    # HUpdate of the smoothing-scale package (SmoothingScaleBase.cc:53-82)
    "total_energy": dict(compatible_energy=False, evolve_total_energy=True),
    "integrate_h": dict(h_update="integrate"),
    "fixed_h": dict(h_update="fixed"),
}


def _make(opts, boundaries="reflecting", two_lists=False):
    p = problems.random_box(n_side=12, seed=81, boundaries=boundaries, two_lists=two_lists)
    p.config.update(opts)
    return p


def _pair(oracle_mod, p, precision="fp64"):
    from spheral_gb300.engine import Engine
    eng = Engine.from_problem(p, precision=precision)
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    return eng, orc


@pytest.mark.parametrize("opt", list(OPTIONS))
def test_option_derivatives_and_steps(native_lib, oracle_mod, opt):
    p = _make(OPTIONS[opt])
    eng, orc = _pair(oracle_mod, p)
    eng.evaluate_derivatives()
    orc.evaluate_derivatives()
    fields = DERIV_FIELDS + (["XSPHWeightSum", "XSPHDeltaV"] if p.config.get("xsph") else [])
    bad = compare_fields(eng, orc, fields, 1e-12)
    assert not bad, bad
    eng2, orc2 = _pair(oracle_mod, _make(OPTIONS[opt]))
    dg, do = eng2.step(), orc2.step()
    assert abs(dg - do) <= 1e-12 * do
    bad = compare_fields(eng2, orc2, STATE_FIELDS, 1e-11)
    assert not bad, bad
    for _ in range(4):
        eng2.step()
        orc2.step()
    bad = compare_fields(eng2, orc2, STATE_FIELDS, 1e-9)
    assert not bad, bad


def test_separate_nodelist_density_sums(native_lib, oracle_mod):
    """sumMassDensityOverAllNodeLists = False with two NodeLists."""
    p = _make(dict(sum_mass_density_over_all_nodelists=False), boundaries="periodic", two_lists=True)
    eng, orc = _pair(oracle_mod, p)
    eng.sum_density()
    orc.sum_density()
    bad = compare_fields(eng, orc, ["massDensity"], 1e-12)
    assert not bad, bad
    eng2, orc2 = _pair(oracle_mod, _make(dict(sum_mass_density_over_all_nodelists=False), boundaries="periodic",
                                         two_lists=True))
    for _ in range(3):
        eng2.step()
        orc2.step()
    bad = compare_fields(eng2, orc2, STATE_FIELDS, 1e-9)
    assert not bad, bad


@pytest.mark.parametrize("h_update", ["integrate", "fixed"])
def test_h_update_steps_mixed(native_lib, oracle_mod, h_update):
    """IntegrateH / FixedH over three mixed-mode steps; FixedH keeps H bitwise."""
    p = _make(dict(h_update=h_update))
    eng, orc = _pair(oracle_mod, p, precision="fp32")
    H0 = eng.field("H")
    for _ in range(3):
        eng.step()
        orc.step()
    bad = compare_fields(eng, orc, ["position", "velocity", "specificThermalEnergy", "H"], 5e-5)
    assert not bad, bad
    if h_update == "fixed":
        assert (eng.field("H") == H0).all()


@pytest.mark.parametrize("opt", ["xsph", "tensile", "no_compatible_energy", "sph_factory_defaults", "total_energy"])
def test_option_mixed_mode(native_lib, oracle_mod, opt):
    p = _make(OPTIONS[opt])
    eng, orc = _pair(oracle_mod, p, precision="fp32")
    eng.evaluate_derivatives()
    orc.evaluate_derivatives()
    fields = ["DvDt", "DepsDt", "DvDx", "massDensitySum", "Hideal"]
    if p.config.get("xsph"):
        fields.append("XSPHDeltaV")
    bad = compare_fields(eng, orc, fields, 5e-5)
    assert not bad, bad
