"""Device-resident SPH engine: a thin Python handle over the C ABI.

``Engine`` owns one ``sphgpu_handle``; the particle state lives on the GPU
between calls and every physics call launches the library's sm_103a kernels.
There is no host fallback: without the built library or a CUDA device every
call raises ``SphGpuError``.
"""
import ctypes

import numpy as np

from . import _native as N

FIELD_NCOMP = {
    "position": 3, "velocity": 3, "mass": 1, "massDensity": 1, "specificThermalEnergy": 1, "H": 6,
    "pressure": 1, "soundSpeed": 1, "omegaGradh": 1, "massDensitySum": 1, "normalization": 1, "DxDt": 3,
    "DvDt": 3, "DrhoDt": 1, "DepsDt": 1, "DvDx": 9, "internalDvDx": 9, "gradRho": 3, "M": 9, "localM": 9,
    "maxViscousPressure": 1, "effViscousPressure": 1, "XSPHWeightSum": 1, "XSPHDeltaV": 3, "DHDt": 6,
    "Hideal": 6, "massZerothMoment": 1, "massFirstMoment": 3, "DvDtGravity": 3, "potential": 1,
    "DepsDtCompatible": 1, "numNeighbors": 1, "ArtificialViscosityVelocityGradient": 9, "massSecondMoment": 6,
    "volume": 1, "rkCorrections": 16,
}

DT_REASONS = ["sound speed", "artificial viscosity", "velocity divergence", "acceleration", "velocity magnitude",
              "pairwise velocity difference", "gravity"]


VISCOSITY = {"monaghan_gingold": 0, "limited_monaghan_gingold": 1}
# smoothing-scale package: SPHSmoothingScale or ASPHClassicSmoothingScale
SMOOTHING_SCALE = {"sph": 0, "asph_classic": 1, "asph": 2}
# HEvolutionType
H_UPDATE = {"ideal": 0, "integrate": 1, "fixed": 2}
# hydro package and the RK volume type of CRKSPH (RKVolumeType)
HYDRO = {"sph": 0, "crksph": 1}
RK_VOLUME = {"mass_over_density": 0, "sum": 1, "h": 4}


def config_from_dict(cfg, precision="fp64", device=0):
    c = N.default_config()
    for k, v in cfg.items():
        if k == "viscosity" and isinstance(v, str):
            c.viscosity = VISCOSITY[v]
        elif k == "smoothing_scale" and isinstance(v, str):
            c.smoothing_scale = SMOOTHING_SCALE[v]
        elif k == "h_update" and isinstance(v, str):
            c.h_update = H_UPDATE[v]
        elif k == "hydro" and isinstance(v, str):
            c.hydro = HYDRO[v]
        elif k == "rk_volume" and isinstance(v, str):
            c.rk_volume = RK_VOLUME[v]
        elif k == "kernel" and isinstance(v, str):
            c.kernel = N.KERNELS[v]
        elif k in dict(N.Config._fields_):
            setattr(c, k, type(getattr(c, k))(v) if not isinstance(v, bool) else int(v))
    c.precision = N.PRECISION[precision] if isinstance(precision, str) else int(precision)
    c.device = device
    return c


class Engine:
    def __init__(self, config=None, precision="fp64", device=0, table=None):
        self.L = N.lib()
        cfg = config_from_dict(config or {}, precision, device)
        self.cfg = cfg
        h = ctypes.c_void_p()
        rc = self.L.sphgpu_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != N.SPHGPU_OK:
            raise N.SphGpuError(rc, "sphgpu_create failed")
        self.h = h
        self.n = 0
        if table is not None:
            self.set_kernel_table(table)

    @classmethod
    def from_problem(cls, problem, precision="fp64", device=0, table=None):
        e = cls(problem.config, precision, device, table)
        e.load(problem)
        return e

    def close(self):
        if getattr(self, "h", None):
            self.L.sphgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        N.check(self.h, rc)

    # -- set up ---------------------------------------------------------------
    def set_kernel_table(self, t):
        arrs = [np.ascontiguousarray(t[k], dtype=np.float64) for k in ("W", "gradW", "grad2W", "nperh", "wsum", "meta")]
        self._table_keep = arrs
        self._chk(self.L.sphgpu_set_kernel_table(self.h, *[N.dptr(a) for a in arrs]))

    def set_nodelist(self, k, nPerh, hmin, hmax, rhoMin, rhoMax, gamma, hminratio=None):
        self._chk(self.L.sphgpu_set_nodelist(self.h, k, nPerh, hmin, hmax, rhoMin, rhoMax, gamma))
        if hminratio is not None:
            self._chk(self.L.sphgpu_set_nodelist_hminratio(self.h, k, hminratio))

    def add_boundary(self, type, axis, lo, hi, wall_high=0):
        self._chk(self.L.sphgpu_add_boundary(self.h, type, axis, lo, hi, wall_high))

    def set_particles(self, pos, vel, mass, rho, eps, H, nodelist=None):
        n = len(mass)
        arr = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        keep = [arr(pos), arr(vel), arr(mass), arr(rho), arr(eps), arr(H)]
        nl = None if nodelist is None else np.ascontiguousarray(nodelist, dtype=np.int32)
        self._chk(self.L.sphgpu_set_particles(self.h, n, *[N.dptr(a) for a in keep],
                                              None if nl is None else N.iptr(nl)))
        self.n = n

    def load(self, problem):
        for k, nl in enumerate(problem.nodelists):
            self.set_nodelist(k, nl["nPerh"], nl["hmin"], nl["hmax"], nl["rhoMin"], nl["rhoMax"], nl["gamma"],
                              nl.get("hminratio"))
        for b in problem.boundaries:
            self.add_boundary(b["type"], b["axis"], b["lo"], b["hi"], b.get("wall_high", 0))
        self.set_particles(problem.pos, problem.vel, problem.mass, problem.rho, problem.eps, problem.H,
                           problem.nodelist)

    # -- physics --------------------------------------------------------------
    def initialize(self):
        self._chk(self.L.sphgpu_initialize(self.h))

    def connectivity(self):
        self._chk(self.L.sphgpu_connectivity(self.h))

    def sum_density(self):
        self._chk(self.L.sphgpu_sum_density(self.h))

    def gradh(self):
        self._chk(self.L.sphgpu_gradh(self.h))

    def evaluate_derivatives(self):
        self._chk(self.L.sphgpu_evaluate_derivatives(self.h))

    def dt(self):
        d = ctypes.c_double()
        r = ctypes.c_int()
        self._chk(self.L.sphgpu_dt(self.h, ctypes.byref(d), ctypes.byref(r)))
        return d.value, (DT_REASONS[r.value] if 0 <= r.value < len(DT_REASONS) else str(r.value))

    def step(self, max_time=1.0e300):
        d = ctypes.c_double()
        rc = self.L.sphgpu_step(self.h, max_time, ctypes.byref(d))
        if rc != N.SPHGPU_OK and getattr(self, "_xerr", None) is not None:
            err, self._xerr = self._xerr, None
            raise N.SphGpuError(rc, "the domain exchange failed: %r" % (err,)) from err
        self._chk(rc)
        return d.value

    def advance(self, nsteps, max_time=1.0e300):
        self._chk(self.L.sphgpu_advance(self.h, nsteps, max_time))

    def synchronize(self):
        self._chk(self.L.sphgpu_synchronize(self.h))

    def checkpoint(self):
        """The restart image of the current state (bytes)."""
        size = ctypes.c_size_t()
        self._chk(self.L.sphgpu_checkpoint_size(self.h, ctypes.byref(size)))
        buf = np.empty(size.value, dtype=np.uint8)
        self._chk(self.L.sphgpu_checkpoint(self.h, buf.ctypes.data, size.value))
        return buf.tobytes()

    def restore(self, image):
        buf = np.frombuffer(image, dtype=np.uint8)
        self._chk(self.L.sphgpu_restore(self.h, buf.ctypes.data, buf.size))
        self.n = int(np.frombuffer(image[16:24], dtype=np.int64)[0])

    def pair_variant(self):
        """(variant in use, number of variants) of the mixed-mode pair kernel."""
        v, nv = ctypes.c_int(), ctypes.c_int()
        self._chk(self.L.sphgpu_get_pair_variant(self.h, ctypes.byref(v), ctypes.byref(nv)))
        return v.value, nv.value

    def neighbor_width(self):
        """Lanes per work group of the neighbour search (autotuned)."""
        w = ctypes.c_int()
        self._chk(self.L.sphgpu_get_neighbor_width(self.h, ctypes.byref(w)))
        return w.value

    def set_pair_variant(self, v):
        self._chk(self.L.sphgpu_set_pair_variant(self.h, v))

    def set_neighbor_width(self, w):
        """Pin the search group width (8, 16 or 32) from the next list build; 0 re-enables the autotuner."""
        self._chk(self.L.sphgpu_set_neighbor_width(self.h, w))

    def energy_variant(self):
        """(batch depth variant in use, number of variants) of the mixed-mode energy sweep."""
        v, nv = ctypes.c_int(), ctypes.c_int()
        self._chk(self.L.sphgpu_get_energy_variant(self.h, ctypes.byref(v), ctypes.byref(nv)))
        return v.value, nv.value

    def set_energy_variant(self, v):
        self._chk(self.L.sphgpu_set_energy_variant(self.h, v))

    @staticmethod
    def ensemble_advance(engines, nsteps, max_time=1.0e300, nthreads=0):
        """nsteps steps of every engine at once (sphgpu_ensemble_advance):
        the boxes run concurrently on their own streams from nthreads host
        threads; each box ends bitwise as if advanced alone."""
        if not engines:
            return
        L = N.lib()
        arr = (ctypes.c_void_p * len(engines))(*[e.h for e in engines])
        failed = ctypes.c_int(-1)
        rc = L.sphgpu_ensemble_advance(arr, len(engines), nsteps, max_time, nthreads, ctypes.byref(failed))
        if rc != N.SPHGPU_OK:
            h = engines[failed.value].h if failed.value >= 0 else None
            N.check(h, rc)

    # -- inspection -----------------------------------------------------------
    def field(self, name):
        nc = FIELD_NCOMP[name]
        out = np.zeros(self.n * nc)
        self._chk(self.L.sphgpu_get_field(self.h, name.encode(), N.dptr(out), None))
        return out.reshape(self.n, nc) if nc > 1 else out

    def set_field(self, name, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._chk(self.L.sphgpu_set_field(self.h, name.encode(), N.dptr(v)))

    def pairs(self):
        n = ctypes.c_long()
        self._chk(self.L.sphgpu_get_pairs(self.h, None, None, None, ctypes.byref(n)))
        i = np.zeros(n.value, np.int32)
        j = np.zeros(n.value, np.int32)
        im = np.zeros(n.value, np.int32)
        self._chk(self.L.sphgpu_get_pairs(self.h, N.iptr(i), N.iptr(j), N.iptr(im), ctypes.byref(n)))
        return i, j, im

    def conservation(self):
        out = np.zeros(8)
        self._chk(self.L.sphgpu_conservation(self.h, N.dptr(out)))
        return out

    @property
    def time(self):
        t = ctypes.c_double()
        self._chk(self.L.sphgpu_get_time(self.h, ctypes.byref(t), None, None))
        return t.value

    def clock(self):
        t, d, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
        self._chk(self.L.sphgpu_get_time(self.h, ctypes.byref(t), ctypes.byref(d), ctypes.byref(c)))
        return t.value, d.value, c.value

    def profile(self, enable=True):
        self._chk(self.L.sphgpu_profile_enable(self.h, 1 if enable else 0))

    def profile_reset(self):
        self._chk(self.L.sphgpu_profile_reset(self.h))

    def profile_get(self, name):
        n = ctypes.c_long()
        ms = ctypes.c_double()
        self._chk(self.L.sphgpu_profile_get(self.h, name.encode(), ctypes.byref(n), ctypes.byref(ms)))
        return n.value, ms.value

    def timer_start(self):
        self._chk(self.L.sphgpu_timer_start(self.h))

    def timer_stop(self):
        ms = ctypes.c_double()
        self._chk(self.L.sphgpu_timer_stop(self.h, ctypes.byref(ms)))
        return ms.value

    def neighbor_entries(self):
        n = ctypes.c_long()
        self._chk(self.L.sphgpu_neighbor_count(self.h, ctypes.byref(n)))
        return n.value

    def upload_state(self, pos=None, vel=None, mass=None, rho=None, eps=None, H=None):
        ptr = lambda a: None if a is None else N.dptr(a)
        self._chk(self.L.sphgpu_upload_state(self.h, ptr(pos), ptr(vel), ptr(mass), ptr(rho), ptr(eps), ptr(H)))

    def download_state(self, pos=None, vel=None, rho=None, eps=None, H=None):
        ptr = lambda a: None if a is None else N.dptr(a)
        self._chk(self.L.sphgpu_download_state(self.h, ptr(pos), ptr(vel), ptr(rho), ptr(eps), ptr(H)))

    # -- domain decomposition -------------------------------------------------
    def set_domain(self, n_ghost, exchange=None):
        """Mark the last n_ghost nodes as halo copies and register
        exchange(point, dt) -> new dt or None, called inside step() at each
        exchange point (see sphgpu_set_domain).  An exception in exchange
        fails the step."""
        if exchange is None:
            self._xcb = None
            self._chk(self.L.sphgpu_set_domain(self.h, int(n_ghost), None, None))
            return

        def cb(user, point, dtp):
            try:
                if point == N.EXCHANGE_DT:
                    dtp[0] = float(exchange(point, float(dtp[0])))
                else:
                    exchange(point, None)
                return 0
            except Exception as e:   # reported through the step's status
                self._xerr = e
                return 1

        self._xerr = None
        self._xcb = N.EXCHANGE_FN(cb)   # kept alive while registered
        self._chk(self.L.sphgpu_set_domain(self.h, int(n_ghost), ctypes.cast(self._xcb, ctypes.c_void_p), None))

    def exchange_width(self, point):
        w = ctypes.c_int()
        self._chk(self.L.sphgpu_exchange_width(self.h, int(point), ctypes.byref(w)))
        return w.value

    def exchange_get(self, point, idx):
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        w = self.exchange_width(point)
        out = np.zeros((len(idx), w))
        if len(idx):
            self._chk(self.L.sphgpu_exchange_get(self.h, int(point), N.iptr(idx), len(idx), N.dptr(out)))
        return out

    def exchange_put(self, point, rows):
        rows = np.ascontiguousarray(rows, dtype=np.float64)
        self._chk(self.L.sphgpu_exchange_put(self.h, int(point), N.dptr(rows)))

    def image_layout(self, field=None):
        """(header bytes, first row of `field` or None, number of rows) of a
        checkpoint image."""
        hb = ctypes.c_size_t()
        row = ctypes.c_int(-1)
        nrows = ctypes.c_int()
        self._chk(self.L.sphgpu_image_layout(self.h, field.encode() if field else None, ctypes.byref(hb),
                                             ctypes.byref(row) if field else None, ctypes.byref(nrows)))
        return hb.value, (row.value if field else None), nrows.value

    def launch_count(self):
        n = ctypes.c_long()
        self._chk(self.L.sphgpu_launch_count(self.h, ctypes.byref(n)))
        return n.value
