"""The Spheral-style scripting front end (spheral_gb300.spheral): names,
defaults and error behaviour, on the CPU (no GPU step is taken)."""
import numpy as np
import pytest

from spheral_gb300 import spheral as S


def test_factory_defaults_follow_the_reference():
    # SPH() defaults (src/SPH/SPHHydros.py:9-33): XSPH on, compatible energy,
    # grad-h, RigorousSumDensity, and LimitedMonaghanGingoldViscosity(1, 1)
    db = S.DataBase()
    W = S.TableKernel(S.BSplineKernel(), 1000)
    hydro = S.SPH(W=W, dataBase=db)
    assert isinstance(hydro.Q, S.LimitedMonaghanGingoldViscosity)
    c = hydro._cfg
    assert c["xsph"] and c["compatible_energy"] and c["gradh_correction"] and c["density_update"] == 0
    assert c["viscosity"] == "limited_monaghan_gingold" and c["eta_crit_frac"] == 1.0 and c["eta_fold_frac"] == 0.2
    nodes = S.makeFluidNodeList("fluid", S.GammaLawGasMKS(5.0 / 3.0, 1.0))
    assert nodes.nodesPerSmoothingScale() == 2.01 and nodes.hmin == 1e-20 and nodes.rhoMin == 1e-10


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
    # with Cl = 2 (extent/4), Cq = (extent/4)^2, no grad-h
    W = S.TableKernel(S.BSplineKernel(), 1000)
    h = S.CRKSPH(dataBase=S.DataBase(), W=W)
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
    h = S.SPH(W=W, dataBase=S.DataBase())
    assert h._cfg["kernel"] == "nbspline" and h._cfg["kernel_order"] == 5
    c = S.CRKSPH(dataBase=S.DataBase(), W=W)
    assert c._cfg["Cl"] == 2.0 * 0.75 and c._cfg["Cq"] == 0.75 ** 2   # Cl = 2 (extent/4), Cq = (extent/4)^2
    with pytest.raises(NotImplementedError):
        S.NBSplineKernel(12)
