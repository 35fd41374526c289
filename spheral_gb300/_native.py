"""ctypes binding of libsphgpu.so (the C ABI declared in include/sphgpu.h).

The library is built in-tree by ``spheral_gb300.build``.  Importing this module
does not touch the GPU; any call that needs the device fails loudly with a
``SphGpuError`` when no CUDA device is present or the library is missing --
there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsphgpu.so")

SPHGPU_OK = 0
ERRORS = {1: "E_CUDA", 2: "E_ARG", 3: "E_UNSUPPORTED", 4: "E_OVERFLOW", 5: "E_NAN", 6: "E_TIMEOUT", 7: "E_STATE"}
PRECISION = {"fp64": 0, "fp32": 1, "fp32_plain": 2}
BOUNDARY_PERIODIC = 0
BOUNDARY_REFLECTING = 1


class SphGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"sphgpu error {ERRORS.get(code, code)}: {msg}")
        self.code = code


class Config(ctypes.Structure):
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
        ("precision", ctypes.c_int),
        ("device", ctypes.c_int),
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


_lib = None

_vp = ctypes.c_void_p
_d = ctypes.c_double
_i = ctypes.c_int
_l = ctypes.c_long
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_long)
_cp = ctypes.c_char_p

SIGNATURES = {
    "sphgpu_default_config": (None, [ctypes.POINTER(Config)]),
    "sphgpu_create": (_i, [ctypes.POINTER(Config), ctypes.POINTER(_vp)]),
    "sphgpu_destroy": (_i, [_vp]),
    "sphgpu_last_error": (_cp, [_vp]),
    "sphgpu_build_bspline_table": (_i, [_i, _dp, _dp, _dp, _dp, _dp, _dp]),
    "sphgpu_build_kernel_table": (_i, [_i, _i, _i, _dp, _dp, _dp, _dp, _dp, _dp]),
    "sphgpu_set_kernel_table": (_i, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "sphgpu_set_nodelist": (_i, [_vp, _i, _d, _d, _d, _d, _d, _d]),
    "sphgpu_set_nodelist_hminratio": (_i, [_vp, _i, _d]),
    "sphgpu_add_boundary": (_i, [_vp, _i, _i, _d, _d, _i]),
    "sphgpu_set_particles": (_i, [_vp, _l, _dp, _dp, _dp, _dp, _dp, _dp, _ip]),
    "sphgpu_initialize": (_i, [_vp]),
    "sphgpu_connectivity": (_i, [_vp]),
    "sphgpu_sum_density": (_i, [_vp]),
    "sphgpu_gradh": (_i, [_vp]),
    "sphgpu_evaluate_derivatives": (_i, [_vp]),
    "sphgpu_dt": (_i, [_vp, _dp, _ip]),
    "sphgpu_step": (_i, [_vp, _d, _dp]),
    "sphgpu_advance": (_i, [_vp, _i, _d]),
    "sphgpu_ensemble_advance": (_i, [_vp, _i, _i, _d, _i, _vp]),
    "sphgpu_set_pair_variant": (_i, [_vp, _i]),
    "sphgpu_checkpoint_size": (_i, [_vp, ctypes.POINTER(ctypes.c_size_t)]),
    "sphgpu_checkpoint": (_i, [_vp, _vp, ctypes.c_size_t]),
    "sphgpu_restore": (_i, [_vp, _vp, ctypes.c_size_t]),
    "sphgpu_get_pair_variant": (_i, [_vp, _ip, _ip]),
    "sphgpu_get_neighbor_width": (_i, [_vp, _ip]),
    "sphgpu_set_neighbor_width": (_i, [_vp, _i]),
    "sphgpu_set_energy_variant": (_i, [_vp, _i]),
    "sphgpu_get_energy_variant": (_i, [_vp, _ip, _ip]),
    "sphgpu_get_field": (_i, [_vp, _cp, _dp, _ip]),
    "sphgpu_set_field": (_i, [_vp, _cp, _dp]),
    "sphgpu_get_pairs": (_i, [_vp, _ip, _ip, _ip, _lp]),
    "sphgpu_upload_state": (_i, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "sphgpu_download_state": (_i, [_vp, _dp, _dp, _dp, _dp, _dp]),
    "sphgpu_conservation": (_i, [_vp, _dp]),
    "sphgpu_get_time": (_i, [_vp, _dp, _dp, _lp]),
    "sphgpu_num_particles": (_i, [_vp, _lp]),
    "sphgpu_profile_enable": (_i, [_vp, _i]),
    "sphgpu_profile_get": (_i, [_vp, _cp, _lp, _dp]),
    "sphgpu_profile_reset": (_i, [_vp]),
    "sphgpu_launch_count": (_i, [_vp, _lp]),
    "sphgpu_synchronize": (_i, [_vp]),
    "sphgpu_timer_start": (_i, [_vp]),
    "sphgpu_timer_stop": (_i, [_vp, _dp]),
    "sphgpu_neighbor_count": (_i, [_vp, _lp]),
    "sphgpu_set_domain": (_i, [_vp, _l, _vp, _vp]),
    "sphgpu_exchange_width": (_i, [_vp, _i, _ip]),
    "sphgpu_exchange_get": (_i, [_vp, _i, _ip, _l, _dp]),
    "sphgpu_exchange_put": (_i, [_vp, _i, _dp]),
    "sphgpu_image_layout": (_i, [_vp, _cp, ctypes.POINTER(ctypes.c_size_t), _ip, _ip]),
}

# Exchange points of sphgpu_set_domain and the callback type.
EXCHANGE_DENSITY, EXCHANGE_DT, EXCHANGE_OMEGA, EXCHANGE_DERIVS = 1, 2, 3, 4
EXCHANGE_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double))


def lib():
    """Load libsphgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SphGpuError(7, f"{LIB_PATH} is missing: run spheral_gb300.build.build() first")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def dptr(a):
    return a.ctypes.data_as(_dp)


def iptr(a):
    return a.ctypes.data_as(_ip)


def check(h, rc):
    if rc != SPHGPU_OK:
        msg = lib().sphgpu_last_error(h) if h else b""
        raise SphGpuError(rc, (msg or b"").decode(errors="replace"))


def default_config():
    c = Config()
    lib().sphgpu_default_config(ctypes.byref(c))
    return c


def build_bspline_table(num_points=1000):
    """Host-side TableKernel(BSplineKernel3d(), num_points) coefficients."""
    nq = num_points | 1
    ncoef = 3 * ((nq - 1) // 2)
    w = np.zeros(ncoef)
    g = np.zeros(ncoef)
    g2 = np.zeros(ncoef)
    nh = np.zeros(2 * num_points)
    ws = np.zeros(2 * num_points)
    meta = np.zeros(9)
    rc = lib().sphgpu_build_bspline_table(num_points, dptr(w), dptr(g), dptr(g2), dptr(nh), dptr(ws), dptr(meta))
    if rc != SPHGPU_OK:
        raise SphGpuError(rc, "build_bspline_table")
    return dict(W=w, gradW=g, grad2W=g2, nperh=nh, wsum=ws, meta=meta)


KERNELS = {"bspline": 0, "nbspline": 1, "wendland_c2": 2, "wendland_c4": 3}


def build_kernel_table(num_points=1000, kernel="bspline", order=3):
    """Host-side TableKernel of a base kernel (BSplineKernel or
    NBSplineKernel(order)); meta[9] is the kernel extent."""
    nq = num_points | 1
    ncoef = 3 * ((nq - 1) // 2)
    w, g, g2 = np.zeros(ncoef), np.zeros(ncoef), np.zeros(ncoef)
    nh, ws, meta = np.zeros(2 * num_points), np.zeros(2 * num_points), np.zeros(10)
    rc = lib().sphgpu_build_kernel_table(KERNELS[kernel] if isinstance(kernel, str) else int(kernel), int(order),
                                         num_points, dptr(w), dptr(g), dptr(g2), dptr(nh), dptr(ws), dptr(meta))
    if rc != SPHGPU_OK:
        raise SphGpuError(rc, "build_kernel_table")
    return dict(W=w, gradW=g, grad2W=g2, nperh=nh, wsum=ws, meta=meta)
