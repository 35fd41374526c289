"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle (``sph_oracle.cpp``) restates the reference's ideal-gas SPH step on
the CPU in FP64 with explicit ghost nodes and an unordered pair list.  Only the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use
this module; the product path never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")


class OrcConfig(ctypes.Structure):
    _fields_ = [
        ("num_table_points", ctypes.c_int),
        ("cfl", ctypes.c_double),
        ("use_velocity_magnitude_for_dt", ctypes.c_int),
        ("compatible_energy", ctypes.c_int),
        ("gradh_correction", ctypes.c_int),
        ("xsph", ctypes.c_int),
        ("correct_velocity_gradient", ctypes.c_int),
        ("sum_mass_density_over_all_nodelists", ctypes.c_int),
        ("density_update", ctypes.c_int),
        ("eps_tensile", ctypes.c_double),
        ("n_tensile", ctypes.c_double),
        ("Cl", ctypes.c_double),
        ("Cq", ctypes.c_double),
        ("eps2", ctypes.c_double),
        ("linear_in_expansion", ctypes.c_int),
        ("quadratic_in_expansion", ctypes.c_int),
        ("dt_min", ctypes.c_double),
        ("dt_max", ctypes.c_double),
        ("dt_growth", ctypes.c_double),
        ("last_dt", ctypes.c_double),
        ("time", ctypes.c_double),
        ("gravity", ctypes.c_int),
        ("G", ctypes.c_double),
        ("softening", ctypes.c_double),
        ("opening", ctypes.c_double),
        ("ftimestep", ctypes.c_double),
        ("viscosity", ctypes.c_int),
        ("eta_crit_frac", ctypes.c_double),
        ("eta_fold_frac", ctypes.c_double),
        ("smoothing_scale", ctypes.c_int),
        ("fix_shape", ctypes.c_int),
        ("h_update", ctypes.c_int),
        ("evolve_total_energy", ctypes.c_int),
        ("radial_only", ctypes.c_int),
        ("hydro", ctypes.c_int),
        ("rk_volume", ctypes.c_int),
        ("kernel", ctypes.c_int),
        ("kernel_order", ctypes.c_int),
    ]


def build(quiet=True):
    """Compile liboracle.so in place (gcc + OpenMP)."""
    out = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(os.path.join(_HERE, "sph_oracle.cpp")):
            build()
        L = ctypes.CDLL(_LIB)
        vp, d, i, l = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_long
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        sig = {
            "orc_create": (vp, [ctypes.POINTER(OrcConfig)]),
            "orc_destroy": (None, [vp]),
            "orc_set_nodelist": (i, [vp, i, d, d, d, d, d, d]),
            "orc_add_boundary": (i, [vp, i, i, d, d, i]),
            "orc_set_particles": (i, [vp, i, dp, dp, dp, dp, dp, dp, ip]),
            "orc_initialize": (i, [vp]),
            "orc_connectivity": (i, [vp]),
            "orc_update_eos": (i, [vp]),
            "orc_sum_density": (i, [vp]),
            "orc_gradh": (i, [vp]),
            "orc_apply_ghosts": (i, [vp]),
            "orc_eval_derivs": (i, [vp]),
            "orc_hydro_dt": (d, [vp]),
            "orc_step": (d, [vp, d]),
            "orc_gravity": (i, [vp]),
            "orc_num_internal": (i, [vp]),
            "orc_num_total": (i, [vp]),
            "orc_num_pairs": (l, [vp]),
            "orc_time": (d, [vp]),
            "orc_get_pairs": (i, [vp, ip, ip, ip]),
            "orc_get_num_neighbors": (i, [vp, ip]),
            "orc_conservation": (None, [vp, dp]),
            "orc_extra_energy": (d, [vp]),
            "orc_dt_min_acc": (d, [vp]),
            "orc_get_field": (i, [vp, ctypes.c_char_p, dp]),
            "orc_set_field": (i, [vp, ctypes.c_char_p, dp]),
            "orc_table": (i, [vp, dp, dp, dp, dp, dp, dp]),
            "orc_kernel_value": (d, [vp, d, d]),
            "orc_grad_value": (d, [vp, d, d]),
            "orc_nperh_lookup": (d, [vp, d]),
            "orc_wsum_lookup": (d, [vp, d]),
            "orc_bspline_value": (d, [d]),
            "orc_bspline_grad": (d, [d]),
            "orc_num_threads": (i, []),
            "orc_set_threads": (i, [i]),
            "orc_set_nodelist_hminratio": (i, [vp, i, d]),
            "orc_sym_eigen": (i, [dp, dp, dp]),
            "orc_smoothing_scale_derivative": (i, [dp, dp, dp]),
            "orc_radial_evolution": (i, [dp, dp, d, d, dp]),
            "orc_rk_volumes": (i, [vp]),
            "orc_nbspline_value": (d, [i, d]),
            "orc_nbspline_grad": (d, [i, d]),
            "orc_rk_corrections": (i, [vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


# artificial viscosity of the SPH package
VISCOSITY = {"monaghan_gingold": 0, "limited_monaghan_gingold": 1}
# smoothing-scale package: SPHSmoothingScale or ASPHClassicSmoothingScale
SMOOTHING_SCALE = {"sph": 0, "asph_classic": 1, "asph": 2}
# HEvolutionType
H_UPDATE = {"ideal": 0, "integrate": 1, "fixed": 2}
# hydro package: SPH or CRKSPH (LinearOrder)
HYDRO = {"sph": 0, "crksph": 1}
# RKVolumeType (RKCorrectionParams.hh): the volume types without a tessellation
RK_VOLUME = {"mass_over_density": 0, "sum": 1, "h": 4}
# base kernel of the TableKernel
KERNEL = {"bspline": 0, "nbspline": 1, "wendland_c2": 2, "wendland_c4": 3}

FIELD_NCOMP = {
    "position": 3, "velocity": 3, "mass": 1, "massDensity": 1, "specificThermalEnergy": 1, "H": 6,
    "pressure": 1, "soundSpeed": 1, "omegaGradh": 1, "massDensitySum": 1, "normalization": 1, "DxDt": 3,
    "DvDt": 3, "DrhoDt": 1, "DepsDt": 1, "DvDx": 9, "internalDvDx": 9, "gradRho": 3, "M": 9, "localM": 9,
    "maxViscousPressure": 1, "effViscousPressure": 1, "XSPHWeightSum": 1, "XSPHDeltaV": 3, "DHDt": 6,
    "Hideal": 6, "massZerothMoment": 1, "massFirstMoment": 3, "DvDtGravity": 3, "potential": 1,
    "DepsDtCompatible": 1, "ArtificialViscosityVelocityGradient": 9, "massSecondMoment": 6,
    "volume": 1, "rkCorrections": 16,
}


class Oracle:
    """One problem instance of the CPU oracle."""

    def __init__(self, problem):
        """``problem`` is a spheral_gb300.problems.Problem-like object with
        ``config`` (dict), ``nodelists``, ``boundaries`` and particle arrays."""
        c = OrcConfig()
        cfg = problem.config
        c.num_table_points = cfg.get("num_table_points", 1000)
        c.cfl = cfg.get("cfl", 0.25)
        c.use_velocity_magnitude_for_dt = int(cfg.get("use_velocity_magnitude_for_dt", False))
        c.compatible_energy = int(cfg.get("compatible_energy", True))
        c.gradh_correction = int(cfg.get("gradh_correction", True))
        c.xsph = int(cfg.get("xsph", False))
        c.correct_velocity_gradient = int(cfg.get("correct_velocity_gradient", True))
        c.sum_mass_density_over_all_nodelists = int(cfg.get("sum_mass_density_over_all_nodelists", True))
        c.density_update = int(cfg.get("density_update", 0))
        c.eps_tensile = cfg.get("eps_tensile", 0.0)
        c.n_tensile = cfg.get("n_tensile", 4.0)
        c.Cl = cfg.get("Cl", 1.0)
        c.Cq = cfg.get("Cq", 1.0)
        c.eps2 = cfg.get("eps2", 1.0e-2)
        c.linear_in_expansion = int(cfg.get("linear_in_expansion", False))
        c.quadratic_in_expansion = int(cfg.get("quadratic_in_expansion", False))
        c.dt_min = cfg.get("dt_min", 0.0)
        c.dt_max = cfg.get("dt_max", 1.0e300)
        c.dt_growth = cfg.get("dt_growth", 2.0)
        c.last_dt = cfg.get("last_dt", 1.0e-5)
        c.time = cfg.get("time", 0.0)
        c.gravity = int(cfg.get("gravity", False))
        c.G = cfg.get("G", 1.0)
        c.softening = cfg.get("softening", 0.01)
        c.opening = cfg.get("opening", 0.5)
        c.ftimestep = cfg.get("ftimestep", 0.1)
        c.viscosity = VISCOSITY[cfg.get("viscosity", "monaghan_gingold")]
        c.eta_crit_frac = cfg.get("eta_crit_frac", 1.0)
        c.eta_fold_frac = cfg.get("eta_fold_frac", 0.2)
        c.smoothing_scale = SMOOTHING_SCALE[cfg.get("smoothing_scale", "sph")]
        c.fix_shape = int(cfg.get("fix_shape", False))
        c.h_update = H_UPDATE[cfg.get("h_update", "ideal")]
        c.evolve_total_energy = int(cfg.get("evolve_total_energy", False))
        c.radial_only = int(cfg.get("radial_only", False))
        c.hydro = HYDRO[cfg.get("hydro", "sph")]
        c.rk_volume = RK_VOLUME[cfg.get("rk_volume", "sum")]
        c.kernel = KERNEL[cfg.get("kernel", "bspline")]
        c.kernel_order = int(cfg.get("kernel_order", 3))
        self._cfg = c
        self.L = lib()
        self.h = self.L.orc_create(ctypes.byref(c))
        for k, nl in enumerate(problem.nodelists):
            self.L.orc_set_nodelist(self.h, k, nl["nPerh"], nl["hmin"], nl["hmax"], nl["rhoMin"], nl["rhoMax"],
                                    nl["gamma"])
            self.L.orc_set_nodelist_hminratio(self.h, k, nl.get("hminratio", 0.1))
        for b in problem.boundaries:
            self.L.orc_add_boundary(self.h, b["type"], b["axis"], b["lo"], b["hi"], b.get("wall_high", 0))
        n = problem.n
        self.n = n
        arr = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self._keep = [arr(problem.pos), arr(problem.vel), arr(problem.mass), arr(problem.rho), arr(problem.eps),
                      arr(problem.H), np.ascontiguousarray(problem.nodelist, dtype=np.int32)]
        k = self._keep
        self.L.orc_set_particles(self.h, n, _dp(k[0]), _dp(k[1]), _dp(k[2]), _dp(k[3]), _dp(k[4]), _dp(k[5]),
                                 _ip(k[6]))

    def __del__(self):
        try:
            self.L.orc_destroy(self.h)
        except Exception:
            pass

    # -- lifecycle --------------------------------------------------------------
    def initialize(self):
        self.L.orc_initialize(self.h)

    def connectivity(self):
        self.L.orc_connectivity(self.h)

    def update_eos(self):
        self.L.orc_update_eos(self.h)

    def sum_density(self):
        self.L.orc_sum_density(self.h)

    def gradh(self):
        self.L.orc_gradh(self.h)

    def rk_volumes(self):
        self.L.orc_rk_volumes(self.h)

    def rk_corrections(self):
        self.L.orc_rk_corrections(self.h)

    def apply_ghosts(self):
        self.L.orc_apply_ghosts(self.h)

    def evaluate_derivatives(self):
        self.L.orc_eval_derivs(self.h)

    def hydro_dt(self):
        return self.L.orc_hydro_dt(self.h)

    def step(self, max_time=1.0e300):
        return self.L.orc_step(self.h, max_time)

    def gravity(self):
        self.L.orc_gravity(self.h)

    # -- inspection -------------------------------------------------------------
    @property
    def time(self):
        return self.L.orc_time(self.h)

    def field(self, name):
        nc = FIELD_NCOMP[name]
        out = np.zeros(self.n * nc, dtype=np.float64)
        r = self.L.orc_get_field(self.h, name.encode(), _dp(out))
        if r < 0:
            raise KeyError(name)
        return out.reshape(self.n, nc) if nc > 1 else out

    def set_field(self, name, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        if self.L.orc_set_field(self.h, name.encode(), _dp(v)) != 0:
            raise KeyError(name)

    def pairs(self):
        """Unordered pair list as (i, j_control, image_code) arrays."""
        n = self.L.orc_num_pairs(self.h)
        i = np.zeros(n, np.int32)
        j = np.zeros(n, np.int32)
        im = np.zeros(n, np.int32)
        self.L.orc_get_pairs(self.h, _ip(i), _ip(j), _ip(im))
        return i, j, im

    def num_neighbors(self):
        out = np.zeros(self.n, np.int32)
        self.L.orc_get_num_neighbors(self.h, _ip(out))
        return out

    def conservation(self):
        out = np.zeros(8, np.float64)
        self.L.orc_conservation(self.h, _dp(out))
        return out

    def extra_energy(self):
        return self.L.orc_extra_energy(self.h)

    def dt_min_acc(self):
        return self.L.orc_dt_min_acc(self.h)

    def table(self):
        npts = self._cfg.num_table_points
        nq = npts + (1 if npts % 2 == 0 else 0)
        ncoef = 3 * ((nq - 1) // 2)
        w = np.zeros(ncoef); g = np.zeros(ncoef); g2 = np.zeros(ncoef)
        nh = np.zeros(2 * npts); ws = np.zeros(2 * npts); meta = np.zeros(10)
        self.L.orc_table(self.h, _dp(w), _dp(g), _dp(g2), _dp(nh), _dp(ws), _dp(meta))
        return dict(W=w, gradW=g, grad2W=g2, nperh=nh, wsum=ws, meta=meta)

    def kernel_value(self, eta, hdet=1.0):
        return self.L.orc_kernel_value(self.h, eta, hdet)

    def grad_value(self, eta, hdet=1.0):
        return self.L.orc_grad_value(self.h, eta, hdet)

    def nperh_lookup(self, wsum):
        return self.L.orc_nperh_lookup(self.h, wsum)

    def wsum_lookup(self, nperh):
        return self.L.orc_wsum_lookup(self.h, nperh)


def bspline_value(eta):
    return lib().orc_bspline_value(eta)


def bspline_grad(eta):
    return lib().orc_bspline_grad(eta)


def num_threads():
    return lib().orc_num_threads()


def set_threads(n):
    """OpenMP threads of the oracle's loops from now on; returns the count."""
    return lib().orc_set_threads(int(n))


def sym_eigen(a6):
    """Eigen-pairs of the symmetric tensor (xx, xy, xz, yy, yz, zz) as the
    oracle's ASPH smoothing scale computes them: (values[3], vectors[3, 3])
    with eigenvector k in column k."""
    a = np.ascontiguousarray(a6, dtype=np.float64)
    vals = np.zeros(3)
    vecs = np.zeros(9)
    lib().orc_sym_eigen(_dp(a), _dp(vals), _dp(vecs))
    return vals, vecs.reshape(3, 3)


def smoothing_scale_derivative(h6, dvdx9):
    """The ASPH tensor DH/Dt of one node."""
    h = np.ascontiguousarray(h6, dtype=np.float64)
    d = np.ascontiguousarray(dvdx9, dtype=np.float64)
    out = np.zeros(6)
    lib().orc_smoothing_scale_derivative(_dp(h), _dp(d), _dp(out))
    return out


def radial_evolution(h6, x3, s, r0):
    """ASPH radialOnly reshaping of one H (the oracle's radialEvolution)."""
    h = np.ascontiguousarray(h6, dtype=np.float64)
    x = np.ascontiguousarray(x3, dtype=np.float64)
    out = np.zeros(6)
    lib().orc_radial_evolution(_dp(h), _dp(x), s, r0, _dp(out))
    return out


def nbspline_value(order, eta):
    """The analytic NBSplineKernel(order) value at eta (Hdet = 1)."""
    return lib().orc_nbspline_value(order, eta)


def nbspline_grad(order, eta):
    return lib().orc_nbspline_grad(order, eta)
