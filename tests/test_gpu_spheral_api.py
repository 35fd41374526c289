"""A Sod-tube script written against the Spheral-style front end runs the
same GPU step as the engine, bitwise."""
import numpy as np
import pytest

from spheral_gb300 import problems
from spheral_gb300 import spheral as S

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
