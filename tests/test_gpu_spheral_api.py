"""A Sod-tube script written against the Spheral-style front end runs the
same GPU step as the engine, bitwise."""
import copy

import numpy as np
import pytest

from spheral_gb300 import problems
from spheral_gb300 import spheral as S

from _parity import DERIV_FIELDS, STATE_FIELDS, compare_fields

pytestmark = pytest.mark.gpu


def _sod_script(nx1=16, ny1=20, steps=5):
    ref = problems.sod(nx1=nx1, ny1=ny1)       # same generator, used for the node data
    W = S.TableKernel(S.BSplineKernel(), 1000)
    eos = S.GammaLawGasMKS(5.0 / 3.0, 1.0)
    nodes = S.makeFluidNodeList("fluid", eos, hmin=1e-10, hmax=1.0, nPerh=1.51, rhoMin=0.01)
    nodes.resize(ref.n)
    nodes.positions()[:] = ref.pos
    nodes.mass()[:] = ref.mass
    nodes.massDensity()[:] = ref.rho
    nodes.specificThermalEnergy()[:] = ref.eps
    nodes.Hfield()[:] = ref.H
    db = S.DataBase()
    db.appendNodeList(nodes)
    q = S.MonaghanGingoldViscosity(1.0, 1.0)
    hydro = S.SPH(W=W, dataBase=db, Q=q, cfl=0.25, XSPH=False)
    L = ref.meta["L"]
    hydro.appendBoundary(S.ReflectingBoundary(S.Plane((0, 0, 0), (1, 0, 0))))
    hydro.appendBoundary(S.ReflectingBoundary(S.Plane((2, 0, 0), (-1, 0, 0))))
    hydro.appendBoundary(S.PeriodicBoundary(S.Plane((0, 0, 0), (0, 1, 0)), S.Plane((0, L, 0), (0, -1, 0))))
    hydro.appendBoundary(S.PeriodicBoundary(S.Plane((0, 0, 0), (0, 0, 1)), S.Plane((0, 0, L), (0, 0, -1))))
    integrator = S.CheapSynchronousRK2Integrator(db, dtMin=1e-6, dtMax=0.1, dtGrowth=2.0)
    integrator.lastDt = 1e-6
    integrator.appendPhysicsPackage(hydro)
    for _ in range(steps):
        integrator.step()
    return ref, nodes, integrator


def test_spheral_style_script_matches_engine(native_lib):
    from spheral_gb300.engine import Engine
    ref, nodes, integrator = _sod_script()
    eng = Engine.from_problem(ref)
    eng.initialize()
    for _ in range(5):
        eng.step()
    assert integrator.currentCycle == 5
    assert integrator.currentTime == eng.time
    assert np.array_equal(nodes.positions(), eng.field("position"))
    assert np.array_equal(nodes.specificThermalEnergy(), eng.field("specificThermalEnergy"))
    assert np.array_equal(nodes.massDensity(), eng.field("massDensity"))


def test_spheral_style_advance_to_goal_time(native_lib):
    ref, nodes, integrator = _sod_script(steps=0)
    n = integrator.advance(0.02)
    assert n > 0 and abs(integrator.currentTime - 0.02) < 1e-14


def test_spheral_style_asph_classic_matches_engine(native_lib):
    # an anisotropic box through SPH(..., ASPH="CLASSIC") runs the same tensor-H step
    from spheral_gb300.engine import Engine
    ref = problems.stretched_box(seed=75)
    W = S.TableKernel(S.BSplineKernel(), 1000)
    nl = ref.nodelists[0]
    nodes = S.makeFluidNodeList("fluid", S.GammaLawGas(5.0 / 3.0), hmin=nl["hmin"], hmax=nl["hmax"],
                                hminratio=nl["hminratio"], nPerh=nl["nPerh"])
    nodes.resize(ref.n)
    nodes.positions()[:] = ref.pos
    nodes.velocity()[:] = ref.vel
    nodes.mass()[:] = ref.mass
    nodes.massDensity()[:] = ref.rho
    nodes.specificThermalEnergy()[:] = ref.eps
    nodes.Hfield()[:] = ref.H
    db = S.DataBase()
    db.appendNodeList(nodes)
    hydro = S.SPH(W=W, dataBase=db, Q=S.MonaghanGingoldViscosity(1.0, 1.0), XSPH=False, ASPH="CLASSIC")
    for a in range(3):
        lo = [0.0, 0.0, 0.0]
        hi = [0.0, 0.0, 0.0]
        hi[a] = 1.0
        nrm = [0.0, 0.0, 0.0]
        nrm[a] = 1.0
        nrm2 = [0.0, 0.0, 0.0]
        nrm2[a] = -1.0
        hydro.appendBoundary(S.PeriodicBoundary(S.Plane(lo, nrm), S.Plane(hi, nrm2)))
    integrator = S.CheapSynchronousRK2Integrator(db, dtMin=0.0, dtMax=0.1, dtGrowth=2.0)
    integrator.lastDt = 1e-3
    integrator.appendPhysicsPackage(hydro)
    for _ in range(3):
        integrator.step()
    eng = Engine.from_problem(ref)
    eng.initialize()
    for _ in range(3):
        eng.step()
    assert np.array_equal(nodes.Hfield(), eng.field("H"))
    assert np.array_equal(nodes.positions(), eng.field("position"))


def test_spheral_style_crksph_matches_engine(native_lib):
    # CRKSPH() with its factory defaults runs the same FP64 CRK step as the engine
    from spheral_gb300.engine import Engine
    ref = problems.crksph_box(n_side=12, seed=57, boundaries="periodic")
    W = S.TableKernel(S.BSplineKernel(), 1000)
    nl = ref.nodelists[0]
    nodes = S.makeFluidNodeList("fluid", S.GammaLawGas(5.0 / 3.0), hmin=nl["hmin"], hmax=nl["hmax"],
                                nPerh=nl["nPerh"])
    nodes.resize(ref.n)
    nodes.positions()[:] = ref.pos
    nodes.velocity()[:] = ref.vel
    nodes.mass()[:] = ref.mass
    nodes.massDensity()[:] = ref.rho
    nodes.specificThermalEnergy()[:] = ref.eps
    nodes.Hfield()[:] = ref.H
    db = S.DataBase()
    db.appendNodeList(nodes)
    hydro = S.CRKSPH(dataBase=db, W=W)
    for a in range(3):
        lo, hi, nrm, nrm2 = [0.0] * 3, [0.0] * 3, [0.0] * 3, [0.0] * 3
        hi[a], nrm[a], nrm2[a] = 1.0, 1.0, -1.0
        hydro.appendBoundary(S.PeriodicBoundary(S.Plane(lo, nrm), S.Plane(hi, nrm2)))
    integrator = S.CheapSynchronousRK2Integrator(db, dtMin=0.0, dtMax=0.1, dtGrowth=2.0)
    integrator.lastDt = 1e-3
    integrator.appendPhysicsPackage(hydro)
    for _ in range(3):
        integrator.step()
    eng = Engine.from_problem(ref)
    eng.initialize()
    for _ in range(3):
        eng.step()
    assert np.array_equal(nodes.positions(), eng.field("position"))
    assert np.array_equal(nodes.specificThermalEnergy(), eng.field("specificThermalEnergy"))


def _periodic_box_script(ref, **sph_kwargs):
    W = S.TableKernel(S.BSplineKernel(), 1000)
    nl = ref.nodelists[0]
    nodes = S.makeFluidNodeList("fluid", S.GammaLawGas(nl["gamma"]), hmin=nl["hmin"], hmax=nl["hmax"],
                                nPerh=nl["nPerh"])
    nodes.resize(ref.n)
    nodes.positions()[:] = ref.pos
    nodes.velocity()[:] = ref.vel
    nodes.mass()[:] = ref.mass
    nodes.massDensity()[:] = ref.rho
    nodes.specificThermalEnergy()[:] = ref.eps
    nodes.Hfield()[:] = ref.H
    db = S.DataBase()
    db.appendNodeList(nodes)
    hydro = S.SPH(W=W, dataBase=db, **sph_kwargs)
    for a in range(3):
        lo, hi, nrm, nrm2 = [0.0] * 3, [0.0] * 3, [0.0] * 3, [0.0] * 3
        hi[a], nrm[a], nrm2[a] = 1.0, 1.0, -1.0
        hydro.appendBoundary(S.PeriodicBoundary(S.Plane(lo, nrm), S.Plane(hi, nrm2)))
    integrator = S.CheapSynchronousRK2Integrator(db, dtMin=0.0, dtMax=0.1, dtGrowth=2.0)
    integrator.lastDt = 1e-3
    integrator.appendPhysicsPackage(hydro)
    return hydro, integrator


def test_sph_factory_default_q_matches_oracle(native_lib, oracle_mod):
    # SPH(W=W, dataBase=db) with no Q builds LimitedMonaghanGingoldViscosity
    # with Cl = 2 (e/2) = 2 and Cq = 2 (e/2)^2 = 2 for NodeLists of extent 2
    # (src/SPH/SPHHydros.py:86-94); the GPU step it drives matches the oracle
    # run with those coefficients: <= 1e-12 after one evaluation, <= 1e-9
    # after five steps.
    ref = problems.random_box(n_side=12, seed=91, boundaries="periodic", vel_scale=0.6)
    hydro, integrator = _periodic_box_script(ref)
    assert isinstance(hydro.Q, S.LimitedMonaghanGingoldViscosity) and hydro.Q.Cl == 2.0 and hydro.Q.Cq == 2.0
    integrator._start()
    prob = integrator._problem
    assert prob.config["viscosity"] == "limited_monaghan_gingold"
    assert prob.config["Cl"] == 2.0 and prob.config["Cq"] == 2.0 and prob.config["xsph"]
    eng = integrator._engine
    orc = oracle_mod.Oracle(prob)
    orc.initialize()
    eng.evaluate_derivatives()
    orc.evaluate_derivatives()
    bad = compare_fields(eng, orc, DERIV_FIELDS + ["XSPHDeltaV"], 1e-12)
    assert not bad, bad
    # the coefficients matter: the oracle with the old (1, 1) differs by far more
    weak = copy.copy(prob)
    weak.config = dict(prob.config, Cl=1.0, Cq=1.0)
    o1 = oracle_mod.Oracle(weak)
    o1.initialize()
    o1.evaluate_derivatives()
    assert compare_fields(eng, o1, ["maxViscousPressure"], 1e-3)
    for _ in range(5):
        integrator.step()
        orc.step()
    bad = compare_fields(eng, orc, STATE_FIELDS, 1e-9)
    assert not bad, bad
