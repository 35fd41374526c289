"""The Spheral-style scripting front end (spheral_gb300.spheral): names,
defaults and error behaviour, on the CPU (no GPU step is taken)."""
import numpy as np
import pytest

from spheral_gb300 import spheral as S


def test_factory_defaults_follow_the_reference():
    # SPH() defaults (src/SPH/SPHHydros.py:9-33): XSPH on, compatible energy,
    # grad-h, RigorousSumDensity, and LimitedMonaghanGingoldViscosity with
    # Cl = 2 (e/2), Cq = 2 (e/2)^2 for e = dataBase.maxKernelExtent (:86-94)
    db = S.DataBase()
    nodes = S.makeFluidNodeList("fluid", S.GammaLawGasMKS(5.0 / 3.0, 1.0))
    assert nodes.nodesPerSmoothingScale() == 2.01 and nodes.hmin == 1e-20 and nodes.rhoMin == 1e-10
    assert nodes.kernelExtent == 2.0
    db.appendNodeList(nodes)
    assert db.maxKernelExtent == 2.0
    W = S.TableKernel(S.BSplineKernel(), 1000)
    hydro = S.SPH(W=W, dataBase=db)
    assert isinstance(hydro.Q, S.LimitedMonaghanGingoldViscosity)
    c = hydro._cfg
    assert c["xsph"] and c["compatible_energy"] and c["gradh_correction"] and c["density_update"] == 0
    assert c["viscosity"] == "limited_monaghan_gingold" and c["eta_crit_frac"] == 1.0 and c["eta_fold_frac"] == 0.2
    assert c["Cl"] == 2.0 and c["Cq"] == 2.0


def test_default_q_follows_the_nodelist_extent():
    # extent 3 (an NBSpline(5) script passes kernelExtent = W.kernelExtent): Cl = 3, Cq = 4.5
    db = S.DataBase()
    db.appendNodeList(S.makeFluidNodeList("a", S.GammaLawGas(5.0 / 3.0), kernelExtent=3.0))
    db.appendNodeList(S.makeFluidNodeList("b", S.GammaLawGas(5.0 / 3.0)))
    assert db.maxKernelExtent == 3.0
    c = S.SPH(W=S.TableKernel(S.NBSplineKernel(5), 1000), dataBase=db)._cfg
    assert c["Cl"] == 3.0 and c["Cq"] == 4.5
    # an empty DataBase has extent 0, so the reference's default Q has no strength
    assert S.DataBase().maxKernelExtent == 0.0
    c0 = S.SPH(W=S.TableKernel(S.BSplineKernel(), 1000), dataBase=S.DataBase())._cfg
    assert c0["Cl"] == 0.0 and c0["Cq"] == 0.0
    # an explicit Q is kept
    q = S.MonaghanGingoldViscosity(1.0, 0.5)
    assert S.SPH(W=S.TableKernel(S.BSplineKernel(), 1000), dataBase=db, Q=q)._cfg["Cq"] == 0.5


def test_nodelist_extent_must_match_the_table_kernel():
    # the GPU neighbour build uses the TableKernel's extent: a NodeList with a
    # different neighbour extent is refused when the integrator starts
    db = S.DataBase()
    nodes = S.makeFluidNodeList("fluid", S.GammaLawGas(5.0 / 3.0), kernelExtent=2.0)
    nodes.resize(8)
    db.appendNodeList(nodes)
    hydro = S.SPH(W=S.TableKernel(S.NBSplineKernel(5), 1000), dataBase=db)
    integ = S.CheapSynchronousRK2Integrator(db)
    integ.appendPhysicsPackage(hydro)
    with pytest.raises(NotImplementedError):
        integ.step()


def test_out_of_path_options_are_refused():
    db = S.DataBase()
    W = S.TableKernel(S.BSplineKernel(), 1000)
    with pytest.raises(NotImplementedError):
        S.SPH(W=W, dataBase=db, ASPH=True)
    with pytest.raises(ValueError):   # SPH.cc:97-98: not with compatible energy
        S.SPH(W=W, dataBase=db, evolveTotalEnergy=True)
    assert S.SPH(W=W, dataBase=db, evolveTotalEnergy=True,
                 compatibleEnergyEvolution=False)._cfg["evolve_total_energy"] is True
    with pytest.raises(NotImplementedError):
        S.TableKernel(object(), 100)
    with pytest.raises(NotImplementedError):
        S.Plane((0, 0, 0), (1, 1, 0))
    with pytest.raises(ValueError):
        S.PeriodicBoundary(S.Plane((0, 0, 0), (1, 0, 0)), S.Plane((1, 0, 0), (1, 0, 0)))


def test_asph_classic_selects_tensor_h():
    # SPH(..., ASPH="CLASSIC") builds ASPHClassicSmoothingScale (SPHHydros.py:130-138)
    db = S.DataBase()
    W = S.TableKernel(S.BSplineKernel(), 1000)
    hydro = S.SPH(W=W, dataBase=db, ASPH="CLASSIC")
    assert isinstance(hydro._smoothingScaleMethod, S.ASPHClassicSmoothingScale)
    assert hydro._cfg["smoothing_scale"] == "asph_classic" and hydro._cfg["fix_shape"] is False
    fixed = S.SPH(W=W, dataBase=db, smoothingScaleMethod=S.ASPHClassicSmoothingScale(S.IdealH, W, fixShape=True))
    assert fixed._cfg["fix_shape"] is True
    assert S.SPH(W=W, dataBase=db)._cfg["smoothing_scale"] == "sph"
    assert S.ASPHClassicSmoothingScale(S.IdealH, W, radialOnly=True)._cfg["radial_only"] is True
    with pytest.raises(ValueError):
        S.ASPHClassicSmoothingScale(S.IdealH, W, fixShape=True, radialOnly=True)
    # HUpdate of the factory maps onto the package
    assert S.SPH(W=W, dataBase=db, HUpdate=S.IntegrateH)._cfg["h_update"] == "integrate"
    assert S.SPH(W=W, dataBase=db, smoothingScaleMethod=S.FixedSmoothingScale())._cfg["h_update"] == "fixed"


def test_boundary_planes_map_to_axis_specs():
    p = S.PeriodicBoundary(S.Plane((0, 0, 0), (0, 1, 0)), S.Plane((0, 2, 0), (0, -1, 0)))
    assert p._spec == dict(type=0, axis=1, lo=0.0, hi=2.0)
    lo = S.ReflectingBoundary(S.Plane((0, 0, 0), (1, 0, 0)))
    hi = S.ReflectingBoundary(S.Plane((3, 0, 0), (-1, 0, 0)))
    assert lo._spec["wall_high"] == 0 and lo._spec["lo"] == 0.0
    assert hi._spec["wall_high"] == 1 and hi._spec["hi"] == 3.0


def test_nodelist_fields_before_the_first_step():
    nodes = S.makeFluidNodeList("fluid", S.GammaLawGas(1.4), nPerh=1.51)
    nodes.resize(10)
    nodes.positions()[:] = np.arange(30).reshape(10, 3)
    assert nodes.positions()[3, 1] == 10.0 and nodes.numInternalNodes == 10


def test_crksph_factory_defaults_follow_the_reference():
    # CRKSPHHydros.py:9-110: XSPH on, compatible energy, LimitedMonaghanGingold
    # with Cl = 2 (e/4), Cq = (e/4)^2 for e = dataBase.maxKernelExtent, no grad-h
    W = S.TableKernel(S.BSplineKernel(), 1000)
    db = S.DataBase()
    db.appendNodeList(S.makeFluidNodeList("fluid", S.GammaLawGas(5.0 / 3.0)))
    h = S.CRKSPH(dataBase=db, W=W)
    c = h._cfg
    assert c["hydro"] == "crksph" and c["rk_volume"] == "sum"
    assert c["xsph"] and c["compatible_energy"] and not c["gradh_correction"]
    assert c["viscosity"] == "limited_monaghan_gingold" and c["Cl"] == 1.0 and c["Cq"] == 0.25
    assert S.CRKSPH(dataBase=S.DataBase(), W=W, volumeType=S.RKMassOverDensity)._cfg["rk_volume"] == "mass_over_density"
    for bad in (dict(order=S.RKOrder.QuadraticOrder), dict(crktype="variant"), dict(ASPH=True),
                dict(volumeType=S.RKVoronoiVolume)):
        with pytest.raises(NotImplementedError):
            S.CRKSPH(dataBase=S.DataBase(), W=W, **bad)
    with pytest.raises(ValueError):
        S.CRKSPH(dataBase=S.DataBase(), W=W, evolveTotalEnergy=True)


def test_nbspline_table_kernel_configures_the_package():
    W = S.TableKernel(S.NBSplineKernel(5), 1000)
    assert W.kernelExtent == 3.0
    db = S.DataBase()
    db.appendNodeList(S.makeFluidNodeList("fluid", S.GammaLawGas(5.0 / 3.0), kernelExtent=W.kernelExtent))
    h = S.SPH(W=W, dataBase=db)
    assert h._cfg["kernel"] == "nbspline" and h._cfg["kernel_order"] == 5
    c = S.CRKSPH(dataBase=db, W=W)
    assert c._cfg["Cl"] == 2.0 * 0.75 and c._cfg["Cq"] == 0.75 ** 2   # Cl = 2 (extent/4), Cq = (extent/4)^2
    with pytest.raises(NotImplementedError):
        S.NBSplineKernel(12)


def test_asph_smoothing_scale_forms():
    # ASPHSmoothingScale (ASPHSmoothingScale.cc): the fixShape and radialOnly
    # forms are on the path, the Voronoi-shaped default form is refused
    W = S.TableKernel(S.BSplineKernel(), 1000)
    db = S.DataBase()
    h = S.SPH(W=W, dataBase=db, smoothingScaleMethod=S.ASPHSmoothingScale(S.IdealH, W, fixShape=True))
    assert h._cfg["smoothing_scale"] == "asph" and h._cfg["fix_shape"] and not h._cfg["radial_only"]
    r = S.SPH(W=W, dataBase=db, smoothingScaleMethod=S.ASPHSmoothingScale(S.IntegrateH, W, radialOnly=True))
    assert r._cfg["radial_only"] and r._cfg["h_update"] == "integrate"
    with pytest.raises(NotImplementedError):
        S.ASPHSmoothingScale(S.IdealH, W)
    with pytest.raises(ValueError):
        S.ASPHSmoothingScale(S.IdealH, W, fixShape=True, radialOnly=True)
