"""CRKSPH (LinearOrder reproducing kernels) on the GPU against the oracle's
restatement (src/CRKSPH/CRKSPH.cc, CRKSPHBase.cc, computeCRKSPHSumMassDensity.cc,
src/RK/RKUtilities.cc, computeRKVolumes.cc, ContinuityVolumePolicy.cc).

Problems: irregular boxes (jittered lattice, mass, energy and h noise, random
velocities) with periodic boundaries, reflecting walls (mirror images carry
the reflected corrections) and open boundaries, for the RK volume types
RKSumVolume, RKMassOverDensity and HVolume; the CRKSPH factory defaults
(XSPH, limited Q with Cl = 1, Cq = 0.25, compatible energy, IdealH).

Tolerances (FP64): neighbour-independent fields after initialize and one
evaluation <= 1e-12 normwise (the 4x4 moment solves use the same LU order
on both sides); one step <= 1e-11, five steps <= 1e-9; linear velocity
fields reproduced to 1e-10; energy conserved to 1e-12.

Mixed mode (FP32 sweeps on the cell-relative mirror, correction moments in
the eta units of each node, FP64 4x4 solves and node completions): volumes,
corrections, density and derivatives <= 1e-5 of the FP64 oracle (measured
<= 2e-6), three steps <= 1e-5 (measured <= 1e-6), dt <= 1e-6, linear
fields reproduced to 1e-5 (measured 3e-7), energy conserved to 1e-9 and
momentum to 1e-9 over five steps (the FP32 pair force is bitwise
antisymmetric; measured ~1e-10).

Long run: the Kelvin-Helmholtz slab in the reference test's CRKSPH setup
(MonaghanGingoldViscosity Cl = Cq = 1, smoothed interfaces) for 300 mixed
steps at 40,000 nodes keeps positive, bounded specific energies and
conserves energy to 1e-8."""
import numpy as np
import pytest

from spheral_gb300 import problems

from _parity import compare_fields

pytestmark = pytest.mark.gpu

STATE = ["position", "velocity", "massDensity", "specificThermalEnergy", "H", "pressure", "soundSpeed", "volume"]
DERIVS = ["DvDt", "DepsDt", "DvDx", "DxDt", "DrhoDt", "XSPHDeltaV", "maxViscousPressure", "effViscousPressure",
          "DHDt", "Hideal", "massZerothMoment", "massFirstMoment"]
CASES = [("periodic", "sum"), ("reflecting", "sum"), ("open", "sum"), ("periodic", "mass_over_density"),
         ("reflecting", "h")]


def _pair(oracle_mod, boundaries, rk_volume, seed=51, **kw):
    from spheral_gb300.engine import Engine
    p = problems.crksph_box(n_side=12, seed=seed, boundaries=boundaries, rk_volume=rk_volume, **kw)
    eng = Engine.from_problem(p, precision="fp64")
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    return p, eng, orc


@pytest.mark.parametrize("boundaries,rk_volume", CASES)
def test_crk_startup_volumes_and_corrections(native_lib, oracle_mod, boundaries, rk_volume):
    p, eng, orc = _pair(oracle_mod, boundaries, rk_volume)
    bad = compare_fields(eng, orc, ["volume", "rkCorrections"], 1e-12)
    assert not bad, bad


@pytest.mark.parametrize("boundaries,rk_volume", CASES)
def test_crk_density_and_derivatives(native_lib, oracle_mod, boundaries, rk_volume):
    p, eng, orc = _pair(oracle_mod, boundaries, rk_volume)
    eng.sum_density()
    orc.sum_density()
    bad = compare_fields(eng, orc, ["massDensity"], 1e-12)
    assert not bad, bad
    eng.evaluate_derivatives()
    orc.rk_corrections()
    orc.evaluate_derivatives()
    bad = compare_fields(eng, orc, DERIVS + ["rkCorrections"], 1e-12)
    assert not bad, bad
    dg, _ = eng.dt()
    assert abs(dg - orc.hydro_dt()) <= 1e-12 * dg


@pytest.mark.parametrize("boundaries,rk_volume", CASES)
def test_crk_step_parity(native_lib, oracle_mod, boundaries, rk_volume):
    p, eng, orc = _pair(oracle_mod, boundaries, rk_volume)
    dg, do = eng.step(), orc.step()
    assert abs(dg - do) <= 1e-12 * do
    bad = compare_fields(eng, orc, STATE, 1e-11)
    assert not bad, bad
    for _ in range(4):
        eng.step()
        orc.step()
    bad = compare_fields(eng, orc, STATE + ["DvDt", "DepsDt", "DvDx", "rkCorrections"], 1e-9)
    assert not bad, bad


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_crk_two_nodelists(native_lib, oracle_mod, precision):
    # two NodeLists: the CRK density sums only the node's own list, XSPH and
    # the moments weight other lists (fweight) as the reference does
    from spheral_gb300.engine import Engine
    p = problems.crksph_box(n_side=12, seed=59, boundaries="periodic", two_lists=True)
    eng = Engine.from_problem(p, precision=precision)
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    tol = 1e-12 if precision == "fp64" else 1e-5
    eng.sum_density()
    orc.sum_density()
    eng.evaluate_derivatives()
    orc.rk_corrections()
    orc.evaluate_derivatives()
    bad = compare_fields(eng, orc, ["massDensity", "DvDt", "DepsDt", "DvDx", "XSPHDeltaV", "Hideal",
                                    "massZerothMoment", "massFirstMoment"], tol)
    assert not bad, bad
    for _ in range(3):
        eng.step()
        orc.step()
    bad = compare_fields(eng, orc, STATE, 1e-10 if precision == "fp64" else 1e-5)
    assert not bad, bad


def test_crk_reproduces_linear_velocity(native_lib, oracle_mod):
    A = np.array([[0.3, -0.2, 0.1], [0.05, -0.4, 0.25], [0.15, 0.2, 0.35]])
    p, eng, orc = _pair(oracle_mod, "open", "sum", seed=53, linear_velocity=A)
    eng.evaluate_derivatives()
    D = eng.field("DvDx").reshape(-1, 3, 3)
    assert np.abs(D - A[None]).max() < 1e-10


@pytest.mark.parametrize("boundaries", ["periodic", "reflecting"])
def test_crk_conserves_and_restarts(native_lib, boundaries):
    from spheral_gb300.engine import Engine
    p = problems.crksph_box(n_side=12, seed=55, boundaries=boundaries)
    eng = Engine.from_problem(p, precision="fp64")
    eng.initialize()
    c0 = eng.conservation()
    eng.advance(3)
    image = eng.checkpoint()
    eng.advance(3)
    c1 = eng.conservation()
    assert abs(c1[7] - c0[7]) <= 1e-12 * abs(c0[7])
    if boundaries == "periodic":
        assert np.abs(c1[1:4] - c0[1:4]).max() <= 1e-12 * np.sqrt(2.0 * c0[0] * c0[4])
    again = Engine(p.config, precision="fp64")
    for k, nl in enumerate(p.nodelists):
        again.set_nodelist(k, nl["nPerh"], nl["hmin"], nl["hmax"], nl["rhoMin"], nl["rhoMax"], nl["gamma"])
    for b in p.boundaries:
        again.add_boundary(b["type"], b["axis"], b["lo"], b["hi"], b.get("wall_high", 0))
    again.restore(image)
    again.advance(3)
    for f in ("position", "velocity", "specificThermalEnergy", "volume"):
        assert np.array_equal(again.field(f), eng.field(f)), f


def _pair_mixed(oracle_mod, boundaries, rk_volume, seed=51, **kw):
    from spheral_gb300.engine import Engine
    p = problems.crksph_box(n_side=12, seed=seed, boundaries=boundaries, rk_volume=rk_volume, **kw)
    eng = Engine.from_problem(p, precision="fp32")
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    return p, eng, orc


@pytest.mark.parametrize("boundaries,rk_volume", CASES)
def test_crk_mixed_evaluation_close(native_lib, oracle_mod, boundaries, rk_volume):
    p, eng, orc = _pair_mixed(oracle_mod, boundaries, rk_volume)
    bad = compare_fields(eng, orc, ["volume", "rkCorrections"], 1e-5)
    assert not bad, bad
    eng.sum_density()
    orc.sum_density()
    bad = compare_fields(eng, orc, ["massDensity"], 1e-5)
    assert not bad, bad
    eng.evaluate_derivatives()
    orc.rk_corrections()
    orc.evaluate_derivatives()
    bad = compare_fields(eng, orc, DERIVS + ["rkCorrections"], 1e-5)
    assert not bad, bad
    dg, _ = eng.dt()
    assert abs(dg - orc.hydro_dt()) <= 1e-6 * dg


@pytest.mark.parametrize("boundaries,rk_volume", CASES)
def test_crk_mixed_steps_close(native_lib, oracle_mod, boundaries, rk_volume):
    p, eng, orc = _pair_mixed(oracle_mod, boundaries, rk_volume)
    for _ in range(3):
        eng.step()
        orc.step()
    bad = compare_fields(eng, orc, STATE + ["DvDt", "DepsDt"], 1e-5)
    assert not bad, bad


def test_crk_mixed_reproduces_linear_velocity(native_lib, oracle_mod):
    A = np.array([[0.3, -0.2, 0.1], [0.05, -0.4, 0.25], [0.15, 0.2, 0.35]])
    p, eng, orc = _pair_mixed(oracle_mod, "open", "sum", seed=53, linear_velocity=A)
    eng.evaluate_derivatives()
    assert np.abs(eng.field("DvDx").reshape(-1, 3, 3) - A[None]).max() < 1e-5


def test_crk_mixed_conserves(native_lib):
    from spheral_gb300.engine import Engine
    p = problems.crksph_box(n_side=12, seed=76, vel_scale=0.1)
    eng = Engine.from_problem(p, precision="fp32")
    eng.initialize()
    c0 = eng.conservation()
    eng.advance(5)
    c1 = eng.conservation()
    assert abs(c1[7] - c0[7]) <= 1e-9 * abs(c0[7])
    assert np.abs(c1[1:4] - c0[1:4]).max() <= 1e-9 * np.sqrt(2.0 * c0[0] * c0[4])


def test_crk_unsupported_settings(native_lib):
    from spheral_gb300 import _native as N
    from spheral_gb300.engine import Engine
    base = problems.crksph_box(n_side=4).config
    with pytest.raises(N.SphGpuError) as e:
        Engine(dict(base, smoothing_scale="asph_classic"), precision="fp64")
    assert e.value.code == 3   # SPHGPU_E_UNSUPPORTED
    with pytest.raises(N.SphGpuError) as e:
        Engine(dict(base, gradh_correction=True), precision="fp64")
    assert e.value.code == 2   # SPHGPU_E_ARG
    with pytest.raises(N.SphGpuError) as e:
        Engine(dict(base, rk_volume=2), precision="fp64")
    assert e.value.code == 3   # SPHGPU_E_UNSUPPORTED


OPTIONS = {
    "integrate_density": dict(density_update=1),
    "total_energy": dict(compatible_energy=False, evolve_total_energy=True),
    "no_xsph": dict(xsph=False),
    "mg_q": dict(viscosity="monaghan_gingold", Cl=1.0, Cq=1.0),
    "integrate_h": dict(h_update="integrate"),
    "fixed_h": dict(h_update="fixed"),
}


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("option", list(OPTIONS))
def test_crk_options(native_lib, oracle_mod, option, precision):
    # the CRKSPH() options on the path: each against the oracle over three steps
    from spheral_gb300.engine import Engine
    p = problems.crksph_box(n_side=12, seed=61, boundaries="reflecting")
    p.config.update(OPTIONS[option])
    eng = Engine.from_problem(p, precision=precision)
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    for _ in range(3):
        eng.step()
        orc.step()
    tol = 1e-10 if precision == "fp64" else 1e-5
    bad = compare_fields(eng, orc, STATE + ["DvDt", "DepsDt"], tol)
    assert not bad, bad


def test_crk_kelvin_helmholtz_long_run(native_lib):
    from spheral_gb300.engine import Engine
    p = problems.kelvin_helmholtz(n1=32, smooth=0.025)
    p.config.update(hydro="crksph", rk_volume="sum", xsph=False, gradh_correction=False,
                    viscosity="monaghan_gingold", Cl=1.0, Cq=1.0)
    eng = Engine.from_problem(p, precision="fp32")
    eng.initialize()
    c0 = eng.conservation()
    eps0 = eng.field("specificThermalEnergy")
    eng.advance(300)
    eps = eng.field("specificThermalEnergy")
    assert eps.min() > 0.5 * eps0.min() and eps.max() < 3.0 * eps0.max(), (eps.min(), eps.max())
    c1 = eng.conservation()
    assert abs(c1[7] - c0[7]) <= 1e-8 * abs(c0[7])
