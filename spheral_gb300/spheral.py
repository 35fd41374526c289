"""Spheral-style scripting front end for the GB300 SPH step.

The classes and factories here carry the names and argument meanings of the
reference's Python layer for this path, so a script written for Spheral's
ideal-gas SPH problem runs on the GPU package with its imports changed:

    TableKernel(BSplineKernel(), numPoints)         src/Kernel/TableKernel.cc:169-209
    GammaLawGasMKS / GammaLawGas(gamma, mu)         src/Material/GammaLawGas.cc
    makeFluidNodeList(name, eos, hmin, hmax, ...)   src/NodeList/FluidNodeLists.py:15-47
    DataBase().appendNodeList(nodes)
    MonaghanGingoldViscosity(Clinear, Cquadratic, ...)         MonaghanGingoldViscosity.cc:25-37
    LimitedMonaghanGingoldViscosity(Clinear, Cquadratic, ..., etaCritFrac, etaFoldFrac)
    SPH(dataBase, W, Q, cfl, ..., XSPH, densityUpdate, epsTensile, nTensile)   src/SPH/SPHHydros.py:9-156
    SPH(..., ASPH="CLASSIC") / ASPHClassicSmoothingScale(HUpdate, W, fixShape)
                                                    src/SmoothingScale/ASPHClassicSmoothingScale.cc
    OctTreeGravity(G, softeningLength, opening, ftimestep)     src/Gravity/TreeGravity.cc:88-115
    Plane(point, normal), PeriodicBoundary(plane1, plane2), ReflectingBoundary(plane)
    CheapSynchronousRK2Integrator(dataBase, dtMin, dtMax, dtGrowth)   src/Integrator/CheapSynchronousRK2.hh
        .appendPhysicsPackage(pkg), .step(maxTime), .advance(goalTime), .currentTime, .lastDt

Node state lives on the GPU once the integrator has taken its first step;
the NodeList accessors (positions(), velocity(), mass(), massDensity(),
specificThermalEnergy(), Hfield()) read it back as numpy arrays.  Only the
ideal-gas SPH path is available: other kernels, EOS, hydro schemes and
boundaries raise NotImplementedError.
"""
import numpy as np

from . import problems
from .engine import Engine

# MassDensityType (src/Hydro/HydroFieldNames / SPH densityUpdate)
RigorousSumDensity = 0
IntegrateDensity = 1
# HEvolutionType (src/SmoothingScale/SmoothingScaleBase.hh:26-30)
IdealH = 0
IntegrateH = 1
FixedH = 2
_H_UPDATE = {IdealH: "ideal", IntegrateH: "integrate", FixedH: "fixed"}


class RKOrder:
    """src/RK/RKCorrectionParams.hh: correction order of the reproducing kernels."""
    ZerothOrder, LinearOrder, QuadraticOrder, CubicOrder = 0, 1, 2, 3
    QuarticOrder, QuinticOrder, SexticOrder, SepticOrder = 4, 5, 6, 7


class RKVolumeType:
    """src/RK/RKCorrectionParams.hh: RK volume weighting."""
    RKMassOverDensity, RKSumVolume, RKVoronoiVolume, RKHullVolume, HVolume = 0, 1, 2, 3, 4


RKMassOverDensity, RKSumVolume, RKVoronoiVolume, RKHullVolume, HVolume = 0, 1, 2, 3, 4
_RK_VOLUME = {RKMassOverDensity: "mass_over_density", RKSumVolume: "sum", HVolume: "h"}


def _h_update(HUpdate):
    if HUpdate not in _H_UPDATE:
        raise NotImplementedError("unknown HEvolutionType")
    return _H_UPDATE[HUpdate]


class SPHSmoothingScale:
    """SPHSmoothingScale(HUpdate, W): isotropic H = I/h (the SPH() default)."""

    def __init__(self, HUpdate=IdealH, W=None):
        self._cfg = dict(smoothing_scale="sph", h_update=_h_update(HUpdate))


class FixedSmoothingScale:
    """FixedSmoothingScale(): H never changes (HEvolutionType FixedH)."""

    def __init__(self):
        self._cfg = dict(smoothing_scale="sph", h_update="fixed")


class ASPHClassicSmoothingScale:
    """ASPHClassicSmoothingScale(HUpdate, W, fixShape=False, radialOnly=False):
    symmetric-tensor H shaped by the second moment of the neighbour
    distribution (src/SmoothingScale/ASPHClassicSmoothingScale.cc); radialOnly
    reshapes H along the radial direction about the origin (the default
    ASPHRadialFunctor)."""

    def __init__(self, HUpdate=IdealH, W=None, fixShape=False, radialOnly=False):
        if fixShape and radialOnly:
            raise ValueError("fixShape and radialOnly cannot both be set")
        self._cfg = dict(smoothing_scale="asph_classic", fix_shape=bool(fixShape), radial_only=bool(radialOnly),
                         h_update=_h_update(HUpdate))


class ASPHSmoothingScale:
    """ASPHSmoothingScale(HUpdate, W, fixShape=False, radialOnly=False)
    (src/SmoothingScale/ASPHSmoothingScale.cc): the tensor H is integrated
    with DH/Dt during the step (IncrementASPHHtensor) and, with IdealH, reset
    at the end of the step from the zeroth moment -- scaled (fixShape) or
    reshaped along the radial direction about the origin (radialOnly).  Its
    default form takes the shape of H from each node's Voronoi cell, a
    tessellation outside this path, and is refused."""

    def __init__(self, HUpdate=IdealH, W=None, fixShape=False, radialOnly=False):
        if fixShape and radialOnly:   # ASPHSmoothingScale.cc:169
            raise ValueError("fixShape and radialOnly cannot both be set")
        if not (fixShape or radialOnly):
            raise NotImplementedError("ASPHSmoothingScale without fixShape or radialOnly shapes H from Voronoi "
                                      "cells, which are not on the GPU path: use fixShape=True, radialOnly=True "
                                      "or ASPH='CLASSIC' (ASPHClassicSmoothingScale)")
        self._cfg = dict(smoothing_scale="asph", fix_shape=bool(fixShape), radial_only=bool(radialOnly),
                         h_update=_h_update(HUpdate))


class BSplineKernel:
    """The cubic B-spline (src/Kernel/BSplineKernelInline.hh:28-93)."""
    kernelExtent = 2.0
    _cfg = dict(kernel="bspline", kernel_order=3)


class NBSplineKernel:
    """The centred cardinal B-spline of a given order
    (src/Kernel/NBSplineKernel.cc:20-118): extent (order + 1) / 2 with the
    reference's integer division, volume normalisation by Simpson's rule."""

    def __init__(self, order):
        order = int(order)
        if not 2 <= order <= 9:
            raise NotImplementedError("NBSplineKernel orders 2..9 are on the GPU path")
        self.order = order
        self.kernelExtent = float((order + 1) // 2)
        self._cfg = dict(kernel="nbspline", kernel_order=order)


class WendlandC2Kernel:
    """Wendland C2, 3-D form (src/Kernel/WendlandC2KernelInline.hh), extent 1."""
    kernelExtent = 1.0
    _cfg = dict(kernel="wendland_c2", kernel_order=0)


class WendlandC4Kernel:
    """Wendland C4, 3-D form (src/Kernel/WendlandC4KernelInline.hh), extent 1."""
    kernelExtent = 1.0
    _cfg = dict(kernel="wendland_c4", kernel_order=0)


class TableKernel:
    def __init__(self, kernel, numPoints=1000):
        if not isinstance(kernel, (BSplineKernel, NBSplineKernel, WendlandC2Kernel, WendlandC4Kernel)):
            raise NotImplementedError("TableKernel of BSplineKernel, NBSplineKernel or WendlandC2/C4Kernel is on "
                                      "the GPU path")
        self.kernel = kernel
        self.numPoints = int(numPoints)
        self.kernelExtent = kernel.kernelExtent


class GammaLawGas:
    def __init__(self, gamma, mu=1.0, constants=None, minimumPressure=None, maximumPressure=None):
        if not gamma > 1.0:
            raise ValueError("gamma must exceed 1")
        self.gamma = float(gamma)
        self.mu = float(mu)


GammaLawGasMKS = GammaLawGas
GammaLawGasCGS = GammaLawGas


class FluidNodeList:
    """The per-NodeList parameters and initial fields of one fluid."""

    def __init__(self, name, eos, numInternal=0, hmin=1.0e-20, hmax=1.0e20, hminratio=0.1, nPerh=2.01,
                 maxNumNeighbors=500, rhoMin=1.0e-10, rhoMax=1e10, kernelExtent=2.0):
        self.name = name
        self.eos = eos
        self.kernelExtent = float(kernelExtent)   # the NodeList's neighbour-search extent
        self.hmin, self.hmax, self.hminratio = float(hmin), float(hmax), float(hminratio)
        self.nPerh = float(nPerh)
        self.rhoMin, self.rhoMax = float(rhoMin), float(rhoMax)
        self._owner = None   # (integrator, index) once the state is on the GPU
        self.numInternalNodes = 0
        self._state = {}
        if numInternal:
            self.resize(numInternal)

    def resize(self, n):
        n = int(n)
        self.numInternalNodes = n
        self._state = dict(position=np.zeros((n, 3)), velocity=np.zeros((n, 3)), mass=np.zeros(n),
                           massDensity=np.zeros(n), specificThermalEnergy=np.zeros(n), H=np.zeros((n, 6)))

    def nodesPerSmoothingScale(self):
        return self.nPerh

    # Field accessors: host arrays before the first step, the GPU state after.
    def _field(self, name):
        if self._owner is not None:
            integ, lo, hi = self._owner
            f = integ._engine.field(name)
            return f[lo:hi] if f.ndim == 1 else f[lo:hi, :]
        return self._state[name]

    def positions(self):
        return self._field("position")

    def velocity(self):
        return self._field("velocity")

    def mass(self):
        return self._field("mass")

    def massDensity(self):
        return self._field("massDensity")

    def specificThermalEnergy(self):
        return self._field("specificThermalEnergy")

    def Hfield(self):
        return self._field("H")

    def pressure(self):
        return self._field("pressure")

    def soundSpeed(self):
        return self._field("soundSpeed")


def makeFluidNodeList(name, eos, numInternal=0, numGhost=0, hmin=1.0e-20, hmax=1.0e20, hminratio=0.1, nPerh=2.01,
                      maxNumNeighbors=500, rhoMin=1.0e-10, rhoMax=1e10, kernelExtent=2.0, **ignored):
    """src/NodeList/FluidNodeLists.py:15-47.  kernelExtent (default 2) is kept:
    DataBase.maxKernelExtent, and through it the SPH()/CRKSPH() default Q,
    depend on it as in the reference.  The other neighbour-object arguments
    are accepted and ignored: the GPU package builds its own cell lists."""
    return FluidNodeList(name, eos, numInternal, hmin, hmax, hminratio, nPerh, maxNumNeighbors, rhoMin, rhoMax,
                         kernelExtent)


class DataBase:
    def __init__(self):
        self.nodeLists = []

    def appendNodeList(self, nodes):
        if not isinstance(nodes, FluidNodeList):
            raise NotImplementedError("only fluid NodeLists are on the GPU path")
        self.nodeLists.append(nodes)

    @property
    def numNodeLists(self):
        return len(self.nodeLists)

    @property
    def maxKernelExtent(self):
        """The largest neighbour-search extent of the NodeLists, 0 with none
        (src/DataBase/DataBase.cc:1742-1748)."""
        return max([nl.kernelExtent for nl in self.nodeLists], default=0.0)

    numFluidNodeLists = numNodeLists


class MonaghanGingoldViscosity:
    kind = "monaghan_gingold"

    def __init__(self, Clinear=1.0, Cquadratic=1.0, kernel=None, linearInExpansion=False,
                 quadraticInExpansion=False):
        self.Cl, self.Cq = float(Clinear), float(Cquadratic)
        self.linearInExpansion = bool(linearInExpansion)
        self.quadraticInExpansion = bool(quadraticInExpansion)
        self.epsilon2 = 1.0e-2

    def _config(self):
        return dict(viscosity=self.kind, Cl=self.Cl, Cq=self.Cq, eps2=self.epsilon2,
                    linear_in_expansion=self.linearInExpansion, quadratic_in_expansion=self.quadraticInExpansion)


class LimitedMonaghanGingoldViscosity(MonaghanGingoldViscosity):
    kind = "limited_monaghan_gingold"

    def __init__(self, Clinear=1.0, Cquadratic=1.0, kernel=None, linearInExpansion=False,
                 quadraticInExpansion=False, etaCritFrac=1.0, etaFoldFrac=0.2):
        super().__init__(Clinear, Cquadratic, kernel, linearInExpansion, quadraticInExpansion)
        self.etaCritFrac, self.etaFoldFrac = float(etaCritFrac), float(etaFoldFrac)

    def _config(self):
        c = super()._config()
        c.update(eta_crit_frac=self.etaCritFrac, eta_fold_frac=self.etaFoldFrac)
        return c


class Plane:
    def __init__(self, point, normal):
        self.point = np.asarray(point, dtype=np.float64)
        self.normal = np.asarray(normal, dtype=np.float64)
        n = self.normal / np.linalg.norm(self.normal)
        axes = np.nonzero(np.abs(n) > 1.0 - 1e-12)[0]
        if len(axes) != 1:
            raise NotImplementedError("only axis-aligned planes are on the GPU path")
        self.axis = int(axes[0])
        self.sign = 1.0 if n[self.axis] > 0 else -1.0


class PeriodicBoundary:
    """PeriodicBoundary(plane1, plane2) between two opposite axis planes."""

    def __init__(self, plane1, plane2):
        if plane1.axis != plane2.axis or plane1.sign == plane2.sign:
            raise ValueError("periodic planes must face each other along one axis")
        lo, hi = sorted((plane1.point[plane1.axis], plane2.point[plane2.axis]))
        self._spec = dict(type=0, axis=plane1.axis, lo=float(lo), hi=float(hi))


class ReflectingBoundary:
    """ReflectingBoundary(plane): a wall at the plane, the fluid on the side
    the normal points to."""

    def __init__(self, plane):
        p = float(plane.point[plane.axis])
        high = plane.sign < 0
        self._spec = dict(type=1, axis=plane.axis, lo=p, hi=p, wall_high=1 if high else 0)


class SPHHydro:
    def __init__(self, dataBase, W, Q, cfl, useVelocityMagnitudeForDt, compatibleEnergyEvolution, gradhCorrection,
                 XSPH, correctVelocityGradient, sumMassDensityOverAllNodeLists, densityUpdate, epsTensile, nTensile,
                 smoothingScaleMethod=None, evolveTotalEnergy=False):
        if compatibleEnergyEvolution and evolveTotalEnergy:   # SPH.cc:97-98
            raise ValueError("SPH error : you cannot simultaneously use both compatibleEnergyEvolution and "
                             "evolveTotalEnergy")
        self.dataBase, self.W, self.Q = dataBase, W, Q
        self.cfl = cfl
        self._cfg = dict(num_table_points=W.numPoints, cfl=cfl,
                         use_velocity_magnitude_for_dt=useVelocityMagnitudeForDt,
                         compatible_energy=compatibleEnergyEvolution, gradh_correction=gradhCorrection,
                         xsph=XSPH, correct_velocity_gradient=correctVelocityGradient,
                         sum_mass_density_over_all_nodelists=sumMassDensityOverAllNodeLists,
                         density_update=densityUpdate, eps_tensile=epsTensile, n_tensile=nTensile,
                         evolve_total_energy=evolveTotalEnergy)
        self._cfg.update(W.kernel._cfg)
        self._cfg.update(Q._config())
        self._smoothingScaleMethod = smoothingScaleMethod or SPHSmoothingScale(IdealH, W)
        self._cfg.update(self._smoothingScaleMethod._cfg)
        self.boundaries = []

    def appendBoundary(self, bc):
        if not isinstance(bc, (PeriodicBoundary, ReflectingBoundary)):
            raise NotImplementedError("only periodic and reflecting planar boundaries are on the GPU path")
        self.boundaries.append(bc)


def SPH(W, WPi=None, WGrad=None, dataBase=None, Q=None, filter=0.0, cfl=0.25, useVelocityMagnitudeForDt=False,
        compatibleEnergyEvolution=True, evolveTotalEnergy=False, gradhCorrection=True, XSPH=True,
        correctVelocityGradient=True, sumMassDensityOverAllNodeLists=True, densityUpdate=RigorousSumDensity,
        HUpdate=IdealH, epsTensile=0.0, nTensile=4.0, damageRelieveRubble=False, strengthInDamage=False,
        xmin=None, xmax=None, etaMinAxis=0.1, ASPH=False, smoothingScaleMethod=None):
    """The SPH() factory (src/SPH/SPHHydros.py:9-156) with its defaults; the
    default Q is LimitedMonaghanGingoldViscosity with Cl = 2 (e/2) and
    Cq = 2 (e/2)^2, e = dataBase.maxKernelExtent (SPHHydros.py:86-94): 2 and 2
    for NodeLists of the default extent 2, 3 and 4.5 for extent 3.
    ASPH="CLASSIC" selects ASPHClassicSmoothingScale (SPHHydros.py:130-138);
    ASPH=True (the Voronoi-based ASPHSmoothingScale) is not on this path."""
    if smoothingScaleMethod is None:
        if ASPH:
            if isinstance(ASPH, str) and ASPH.upper() == "CLASSIC":
                smoothingScaleMethod = ASPHClassicSmoothingScale(HUpdate, W)
            else:
                smoothingScaleMethod = ASPHSmoothingScale(HUpdate, W)
        else:
            smoothingScaleMethod = SPHSmoothingScale(HUpdate, W)
    elif not isinstance(smoothingScaleMethod, (SPHSmoothingScale, ASPHClassicSmoothingScale, ASPHSmoothingScale,
                                               FixedSmoothingScale)):
        raise NotImplementedError("unknown smoothing-scale package")
    if (filter or 0.0) != 0.0:
        raise NotImplementedError("H filtering is not on the GPU path")
    if not Q:
        e = dataBase.maxKernelExtent / 2.0
        Q = LimitedMonaghanGingoldViscosity(2.0 * e, 2.0 * e * e)
    return SPHHydro(dataBase, W, Q, cfl, useVelocityMagnitudeForDt, compatibleEnergyEvolution, gradhCorrection,
                    XSPH, correctVelocityGradient, sumMassDensityOverAllNodeLists, densityUpdate, epsTensile,
                    nTensile, smoothingScaleMethod, evolveTotalEnergy)


class CRKSPHHydro(SPHHydro):
    """CRKSPH package (src/CRKSPH/CRKSPH.cc) with its RKCorrections companion
    (src/RK/RKCorrections.cc) at LinearOrder, in FP64."""

    def __init__(self, dataBase, W, Q, cfl, useVelocityMagnitudeForDt, compatibleEnergyEvolution, evolveTotalEnergy,
                 XSPH, densityUpdate, epsTensile, nTensile, smoothingScaleMethod, volumeType):
        if compatibleEnergyEvolution and evolveTotalEnergy:   # CRKSPH.cc:99-101
            raise ValueError("CRKSPH error : you cannot simultaneously use both compatibleEnergyEvolution and "
                             "evolveTotalEnergy")
        if volumeType not in _RK_VOLUME:
            raise NotImplementedError("RKVoronoiVolume and RKHullVolume need a tessellation and are not on the "
                                      "GPU path")
        super().__init__(dataBase, W, Q, cfl, useVelocityMagnitudeForDt, compatibleEnergyEvolution, False, XSPH,
                         False, True, densityUpdate, epsTensile, nTensile, smoothingScaleMethod, evolveTotalEnergy)
        self._cfg.update(hydro="crksph", rk_volume=_RK_VOLUME[volumeType])


def CRKSPH(dataBase, W, Q=None, order=RKOrder.LinearOrder, filter=0.0, cfl=0.25, useVelocityMagnitudeForDt=False,
           compatibleEnergyEvolution=True, evolveTotalEnergy=False, XSPH=True, densityUpdate=RigorousSumDensity,
           HUpdate=IdealH, epsTensile=0.0, nTensile=4.0, damageRelieveRubble=False, ASPH=False, etaMinAxis=0.1,
           crktype="default", smoothingScaleMethod=None, volumeType=RKSumVolume):
    """The CRKSPH() factory (src/CRKSPH/CRKSPHHydros.py:9-110) with its
    defaults: the default Q is LimitedMonaghanGingoldViscosity with
    Cl = 2 (e/4) and Cq = (e/4)^2, e = dataBase.maxKernelExtent
    (CRKSPHHydros.py:64-68).  The reference hands the RK
    volume type to SpheralController (default RKVoronoiVolume, which needs a
    tessellation); here it is the volumeType argument, RKSumVolume by default.
    LinearOrder, the default crktype and SPHSmoothingScale are on this path."""
    if order != RKOrder.LinearOrder:
        raise NotImplementedError("only LinearOrder reproducing kernels are on the GPU path")
    if crktype.lower() != "default":
        raise NotImplementedError("CRKSPHVariant is not on the GPU path")
    if ASPH:
        raise NotImplementedError("ACRKSPH is not on the GPU path")
    if smoothingScaleMethod is None:
        smoothingScaleMethod = SPHSmoothingScale(HUpdate, W)
    elif not isinstance(smoothingScaleMethod, (SPHSmoothingScale, FixedSmoothingScale)):
        raise NotImplementedError("CRKSPH runs with SPHSmoothingScale on the GPU path")
    if not Q:
        e = dataBase.maxKernelExtent / 4.0
        Q = LimitedMonaghanGingoldViscosity(2.0 * e, e * e)
    return CRKSPHHydro(dataBase, W, Q, cfl, useVelocityMagnitudeForDt, compatibleEnergyEvolution, evolveTotalEnergy,
                       XSPH, densityUpdate, epsTensile, nTensile, smoothingScaleMethod, volumeType)


class OctTreeGravity:
    def __init__(self, G, softeningLength, opening=0.5, ftimestep=0.1, timeStepChoice=None):
        self._cfg = dict(gravity=True, G=float(G), softening=float(softeningLength), opening=float(opening),
                         ftimestep=float(ftimestep))


class CheapSynchronousRK2Integrator:
    """CheapSynchronousRK2 over the GPU package: step(maxTime) advances one
    cycle, advance(goalTime) steps until goalTime."""

    def __init__(self, dataBase, dtMin=0.0, dtMax=1.0e300, dtGrowth=2.0, precision="fp64"):
        self.dataBase = dataBase
        self.dtMin, self.dtMax, self.dtGrowth = float(dtMin), float(dtMax), float(dtGrowth)
        self.lastDt = 1.0e-5
        self.precision = precision
        self.packages = []
        self._engine = None
        self._cycle = 0

    def appendPhysicsPackage(self, pkg):
        if not isinstance(pkg, (SPHHydro, OctTreeGravity)):
            raise NotImplementedError("only SPH and OctTreeGravity are on the GPU path")
        self.packages.append(pkg)

    def _start(self):
        hydros = [p for p in self.packages if isinstance(p, SPHHydro)]
        if len(hydros) != 1:
            raise RuntimeError("exactly one SPH package is needed")
        hydro = hydros[0]
        cfg = dict(hydro._cfg)
        for p in self.packages:
            if isinstance(p, OctTreeGravity):
                cfg.update(p._cfg)
        cfg.update(dt_min=self.dtMin, dt_max=self.dtMax, dt_growth=self.dtGrowth, last_dt=self.lastDt)
        lists = self.dataBase.nodeLists
        if not lists:
            raise RuntimeError("the DataBase has no NodeLists")
        for nl in lists:
            # the GPU neighbour build takes its extent from the TableKernel; the
            # reference takes the NodeLists' (ConnectivityMap.cc:779-786)
            if nl.kernelExtent != hydro.W.kernelExtent:
                raise NotImplementedError(f"NodeList {nl.name!r} has kernelExtent {nl.kernelExtent}, the TableKernel "
                                          f"{hydro.W.kernelExtent}: the GPU path needs them equal")
        pieces = [nl._state for nl in lists]
        cat = lambda k: np.concatenate([p[k] for p in pieces])
        H = cat("H")
        nodelist = np.concatenate([np.full(nl.numInternalNodes, k, dtype=np.int32) for k, nl in enumerate(lists)])
        nls = [dict(nPerh=nl.nPerh, hmin=nl.hmin, hmax=nl.hmax, rhoMin=nl.rhoMin, rhoMax=nl.rhoMax,
                    gamma=nl.eos.gamma, hminratio=nl.hminratio) for nl in lists]
        prob = problems.Problem("script", cat("position"), cat("velocity"), cat("mass"), cat("massDensity"),
                                cat("specificThermalEnergy"), 1.0 / H[:, 0], nodelist if len(lists) > 1 else None,
                                nls, [b._spec for b in hydro.boundaries], cfg)
        prob.H = np.ascontiguousarray(H)
        self._problem = prob
        self._engine = Engine.from_problem(prob, precision=self.precision)
        self._engine.initialize()
        lo = 0
        for nl in lists:
            nl._owner = (self, lo, lo + nl.numInternalNodes)
            lo += nl.numInternalNodes

    def step(self, maxTime=1.0e300):
        if self._engine is None:
            self._start()
        dt = self._engine.step(maxTime)
        self.lastDt = dt
        self._cycle += 1
        return True

    def advance(self, goalTime, maxSteps=None):
        n = 0
        while self.currentTime < goalTime * (1.0 - 1e-15) and (maxSteps is None or n < maxSteps):
            self.step(goalTime)
            n += 1
        return n

    @property
    def currentTime(self):
        return 0.0 if self._engine is None else self._engine.time

    @property
    def currentCycle(self):
        return self._cycle
