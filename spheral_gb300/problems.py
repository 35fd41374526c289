"""Seeded synthetic problems for the SPH hot path.

Each generator returns a :class:`Problem` with isotropic H = I/h (h = nPerh
times the local lattice spacing), GammaLawGas internal energies from the
stated pressure, NodeList parameters, boundaries and package settings.  They
stand in for the reference's functional setups (no external data is read):

* :func:`sod`      -- planar Sod tube of tests/functional/Hydro/Sod/Sod-planar-3d.py
                      (left lattice dx, right lattice 2dx with twice the mass).
* :func:`kelvin_helmholtz` -- periodic KH slab of
                      tests/functional/Hydro/KelvinHelmholtz/KelvinHelmholtz-3d.py,
                      two equal-mass-ish lattices with spacing ratio ~2^(-1/3).
* :func:`evrard`   -- rho ~ 1/r sphere of
                      tests/functional/EvrardSphericalCollapse/EvrardSphericalCollapse.py.
* :func:`turbulent_box` / :func:`ensemble` -- periodic boxes with a k^-4
                      Gaussian velocity field (batched ensemble workload).
* :func:`sweep_box` -- jittered periodic lattice with a chosen neighbour count.
"""
import math

import numpy as np

GAMMA = 5.0 / 3.0


def nperh_for_neighbors(k):
    """nPerh giving a mean gather count k for the extent-2 B-spline:
    k = (4 pi / 3) (2 nPerh)^3."""
    return 0.5 * (3.0 * k / (4.0 * math.pi)) ** (1.0 / 3.0)


class Problem:
    def __init__(self, name, pos, vel, mass, rho, eps, h, nodelist=None, nodelists=None, boundaries=None,
                 config=None, meta=None):
        self.name = name
        self.pos = np.ascontiguousarray(pos, dtype=np.float64)
        self.vel = np.ascontiguousarray(vel, dtype=np.float64)
        self.mass = np.ascontiguousarray(mass, dtype=np.float64)
        self.rho = np.ascontiguousarray(rho, dtype=np.float64)
        self.eps = np.ascontiguousarray(eps, dtype=np.float64)
        n = len(self.mass)
        hinv = 1.0 / np.asarray(h, dtype=np.float64)
        H = np.zeros((n, 6))
        H[:, 0] = hinv
        H[:, 3] = hinv
        H[:, 5] = hinv
        self.H = H
        self.nodelist = np.zeros(n, np.int32) if nodelist is None else np.ascontiguousarray(nodelist, np.int32)
        self.nodelists = nodelists or [dict(nPerh=1.51, hmin=1e-20, hmax=1e20, rhoMin=1e-10, rhoMax=1e10,
                                            gamma=GAMMA)]
        self.boundaries = boundaries or []
        self.config = dict(config or {})
        self.meta = dict(meta or {})

    @property
    def n(self):
        return len(self.mass)

    def copy(self):
        p = Problem(self.name, self.pos.copy(), self.vel.copy(), self.mass.copy(), self.rho.copy(), self.eps.copy(),
                    1.0 / self.H[:, 0], self.nodelist.copy(), [dict(d) for d in self.nodelists],
                    [dict(b) for b in self.boundaries], dict(self.config), dict(self.meta))
        p.H = self.H.copy()
        return p


def _lattice(nx, ny, nz, lo, hi):
    xs = lo[0] + (np.arange(nx) + 0.5) * (hi[0] - lo[0]) / nx
    ys = lo[1] + (np.arange(ny) + 0.5) * (hi[1] - lo[1]) / ny
    zs = lo[2] + (np.arange(nz) + 0.5) * (hi[2] - lo[2]) / nz
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)


def periodic_box_boundaries(lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), axes=(0, 1, 2)):
    return [dict(type=0, axis=a, lo=lo[a], hi=hi[a]) for a in axes]


def sod(nx1=80, ny1=20, nPerh=1.51, cfl=0.25):
    """3-D planar Sod tube: x in [0, 2] split at x = 1, y, z in [0, L] periodic
    with L = ny1/nx1, reflecting walls at x = 0 and x = 2.  The left lattice
    has spacing dx = 1/nx1 (rho = 1, P = 1); the right lattice 2 dx with twice
    the particle mass (rho = 0.25, P = 0.1795).  nx1 = 80 gives
    80x20x20 + 40x10x10 = 36,000 nodes."""
    dx1 = 1.0 / nx1
    L = ny1 * dx1
    left = _lattice(nx1, ny1, ny1, (0.0, 0.0, 0.0), (1.0, L, L))
    right = _lattice(nx1 // 2, ny1 // 2, ny1 // 2, (1.0, 0.0, 0.0), (2.0, L, L))
    pos = np.concatenate([left, right])
    nl, nr = len(left), len(right)
    dx2 = 2.0 * dx1
    rho = np.concatenate([np.full(nl, 1.0), np.full(nr, 0.25)])
    P = np.concatenate([np.full(nl, 1.0), np.full(nr, 0.1795)])
    mass = np.concatenate([np.full(nl, 1.0 * dx1 ** 3), np.full(nr, 0.25 * dx2 ** 3)])
    h = np.concatenate([np.full(nl, nPerh * dx1), np.full(nr, nPerh * dx2)])
    eps = P / ((GAMMA - 1.0) * rho)
    bcs = [dict(type=1, axis=0, lo=0.0, hi=2.0, wall_high=0), dict(type=1, axis=0, lo=0.0, hi=2.0, wall_high=1),
           dict(type=0, axis=1, lo=0.0, hi=L), dict(type=0, axis=2, lo=0.0, hi=L)]
    cfg = dict(cfl=cfl, compatible_energy=True, gradh_correction=True, xsph=False, correct_velocity_gradient=True,
               Cl=1.0, Cq=1.0, dt_min=1.0e-6, dt_max=0.1, dt_growth=2.0, last_dt=1.0e-6)
    nls = [dict(nPerh=nPerh, hmin=1e-10, hmax=1.0, rhoMin=0.01, rhoMax=1e10, gamma=GAMMA)]
    return Problem("sod", pos, np.zeros_like(pos), mass, rho, eps, h, None, nls, bcs, cfg,
                   meta=dict(nx1=nx1, ny1=ny1, L=L))


def kelvin_helmholtz(n1=112, n2=None, jitter=0.05, seed=1, nPerh=1.51, smooth=0.0):
    """Periodic unit-cube Kelvin-Helmholtz slab: |y - 0.5| < 0.25 has rho = 2,
    vx = +0.5 on a lattice of n2 per unit length; outside rho = 1, vx = -0.5
    on n1 per unit length; vy = 0.01 sin(4 pi x); P = 2.5.  n2 defaults to the
    even integer nearest n1 2^(1/3) (spacing ratio ~2^(-1/3), near-equal
    masses set so the densities are exact).  Positions get Gaussian jitter of
    jitter x spacing (seed).

    smooth > 0 tapers density and shear velocity across the two interfaces
    as the reference's own 3-D test does
    (tests/functional/Hydro/KelvinHelmholtz/KelvinHelmholtz-3d.py:246-270):
    at distance d from the nearest interface the jump is relaxed by
    exp(-d / smooth) from each side towards the mean (rho 1.5, vx 0), node
    masses follow rho / rho_nominal and the energies keep P = 2.5."""
    if n2 is None:
        n2 = int(round(n1 * 2.0 ** (1.0 / 3.0) / 2.0)) * 2
    rng = np.random.default_rng(seed)
    d1, d2 = 1.0 / n1, 1.0 / n2
    lowr = _lattice(n1, n1 // 4, n1, (0.0, 0.0, 0.0), (1.0, 0.25, 1.0))
    highr = _lattice(n1, n1 // 4, n1, (0.0, 0.75, 0.0), (1.0, 1.0, 1.0))
    slab = _lattice(n2, n2 // 2, n2, (0.0, 0.25, 0.0), (1.0, 0.75, 1.0))
    outer = np.concatenate([lowr, highr])
    no, ns = len(outer), len(slab)
    outer = outer + rng.normal(0.0, jitter * d1, outer.shape)
    slab = slab + rng.normal(0.0, jitter * d2, slab.shape)
    pos = np.mod(np.concatenate([outer, slab]), 1.0)
    rho = np.concatenate([np.full(no, 1.0), np.full(ns, 2.0)])
    mass = np.concatenate([np.full(no, 0.5 / no), np.full(ns, 1.0 / ns)])
    h = np.concatenate([np.full(no, nPerh * d1), np.full(ns, nPerh * d2)])
    vel = np.zeros_like(pos)
    vel[:no, 0] = -0.5
    vel[no:, 0] = 0.5
    vel[:, 1] = 0.01 * np.sin(4.0 * math.pi * pos[:, 0])
    if smooth > 0.0:
        d = np.minimum(np.abs(pos[:, 1] - 0.25), np.abs(pos[:, 1] - 0.75))
        f = 0.5 * np.exp(-d / smooth)
        sign = np.concatenate([np.full(no, 1.0), np.full(ns, -1.0)])   # outer rises, slab falls
        new = rho + sign * f
        mass = mass * new / rho
        rho = new
        vel[:, 0] += sign * f
    eps = 2.5 / ((GAMMA - 1.0) * rho)
    cfg = dict(cfl=0.5, compatible_energy=True, gradh_correction=False, xsph=False, correct_velocity_gradient=True,
               Cl=1.0, Cq=1.0, dt_min=1.0e-8, dt_max=0.1, dt_growth=2.0, last_dt=1.0e-4)
    nls = [dict(nPerh=nPerh, hmin=1e-4, hmax=0.5, rhoMin=1e-10, rhoMax=1e10, gamma=GAMMA)]
    return Problem("kelvin_helmholtz", pos, vel, mass, rho, eps, h, None, nls, periodic_box_boundaries(), cfg,
                   meta=dict(n1=n1, n2=n2, seed=seed, smooth=smooth))


def evrard(n=1048576, seed=2, nPerh=1.51, G=1.0, softening=0.01, opening=0.5):
    """Evrard collapse: n equal-mass nodes in the unit sphere with rho ~ 1/r
    (r = U^(1/2), isotropic directions, seed), total mass 1, u = 0.05, v = 0,
    G = 1, TreeGravity opening 0.5 and Plummer softening 0.01."""
    rng = np.random.default_rng(seed)
    r = np.sqrt(rng.random(n))
    mu = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * math.pi, n)
    s = np.sqrt(1.0 - mu * mu)
    pos = np.stack([r * s * np.cos(phi), r * s * np.sin(phi), r * mu], axis=1)
    m = np.full(n, 1.0 / n)
    rho0 = 1.0 / (2.0 * math.pi)
    rho = rho0 / np.maximum(r, 1e-6)
    h = nPerh * (m / rho) ** (1.0 / 3.0)
    eps = np.full(n, 0.05)
    cfg = dict(cfl=0.5, compatible_energy=True, gradh_correction=True, xsph=False, correct_velocity_gradient=True,
               Cl=1.0, Cq=1.0, dt_min=1.0e-8, dt_max=0.1, dt_growth=2.0, last_dt=1.0e-5, gravity=True, G=G,
               softening=softening, opening=opening, ftimestep=0.1)
    nls = [dict(nPerh=nPerh, hmin=1e-10, hmax=10.0, rhoMin=1e-10, rhoMax=1e10, gamma=GAMMA)]
    return Problem("evrard", pos, np.zeros_like(pos), m, rho, eps, h, None, nls, [], cfg, meta=dict(seed=seed))


def _k4_velocity_field(n, seed, mach=0.3, cs=math.sqrt(GAMMA * 1.0 / 1.0)):
    """Gaussian random velocity field on an n^3 periodic grid with power
    spectrum P(k) ~ k^-4, rescaled to rms speed mach * cs."""
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(n) * n
    KX, KY, KZ = np.meshgrid(k, k, k, indexing="ij")
    k2 = KX * KX + KY * KY + KZ * KZ
    k2[0, 0, 0] = 1.0
    amp = k2 ** (-1.0)       # |v_k| ~ sqrt(P(k)) ~ k^-2
    amp[0, 0, 0] = 0.0
    v = []
    for _ in range(3):
        noise = rng.normal(size=(n, n, n)) + 1j * rng.normal(size=(n, n, n))
        v.append(np.real(np.fft.ifftn(noise * amp)))
    v = np.stack([c.ravel() for c in v], axis=1)
    v -= v.mean(axis=0)
    rms = np.sqrt(np.mean(np.sum(v * v, axis=1)))
    return v * (mach * cs / rms)


def turbulent_box(n_side, seed, nPerh=1.51, mach=0.3):
    """Periodic unit cube, n_side^3 lattice, rho = 1, P = 1, k^-4 velocities."""
    pos = _lattice(n_side, n_side, n_side, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    n = len(pos)
    d = 1.0 / n_side
    rho = np.ones(n)
    mass = np.full(n, d ** 3)
    h = np.full(n, nPerh * d)
    eps = np.full(n, 1.0 / ((GAMMA - 1.0) * 1.0))
    vel = _k4_velocity_field(n_side, seed, mach)
    cfg = dict(cfl=0.25, compatible_energy=True, gradh_correction=True, xsph=False, correct_velocity_gradient=True,
               Cl=1.0, Cq=1.0, dt_min=1.0e-8, dt_max=0.1, dt_growth=2.0, last_dt=1.0e-4)
    nls = [dict(nPerh=nPerh, hmin=1e-6, hmax=0.5, rhoMin=1e-10, rhoMax=1e10, gamma=GAMMA)]
    return Problem("turbulent_box", pos, vel, mass, rho, eps, h, None, nls, periodic_box_boundaries(), cfg,
                   meta=dict(n_side=n_side, seed=seed))


def ensemble_sizes(nboxes=256, seed=3, nmin=4096, nmax=262144):
    """Box particle counts, log-uniform in [nmin, nmax] (seed), each rounded to
    the nearest cube n^3."""
    rng = np.random.default_rng(seed)
    nb = np.exp(rng.uniform(math.log(nmin), math.log(nmax), nboxes))
    return [int(round(x ** (1.0 / 3.0))) for x in nb]


def ensemble(nboxes=256, seed=3, nmin=4096, nmax=262144):
    return [turbulent_box(s, 4 + b) for b, s in enumerate(ensemble_sizes(nboxes, seed, nmin, nmax))]


def sweep_box(n_side=256, neighbors=64, seed=5, jitter=0.1):
    """Periodic unit cube lattice, Gaussian jitter jitter x spacing, rho = 1
    with 1% uniform noise (through the mass), P = 1, v ~ N(0, 0.1)."""
    rng = np.random.default_rng(seed)
    nPerh = nperh_for_neighbors(neighbors)
    d = 1.0 / n_side
    pos = _lattice(n_side, n_side, n_side, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    n = len(pos)
    pos = np.mod(pos + rng.normal(0.0, jitter * d, pos.shape), 1.0)
    rho = 1.0 + 0.01 * rng.uniform(-1.0, 1.0, n)
    mass = rho * d ** 3
    h = np.full(n, nPerh * d)
    eps = 1.0 / ((GAMMA - 1.0) * rho)
    vel = rng.normal(0.0, 0.1, (n, 3))
    cfg = dict(cfl=0.25, compatible_energy=True, gradh_correction=True, xsph=False, correct_velocity_gradient=True,
               Cl=1.0, Cq=1.0, dt_min=1.0e-8, dt_max=0.1, dt_growth=2.0, last_dt=1.0e-4)
    nls = [dict(nPerh=nPerh, hmin=1e-6, hmax=0.5, rhoMin=1e-10, rhoMax=1e10, gamma=GAMMA)]
    return Problem("sweep_box", pos, vel, mass, rho, eps, h, None, nls, periodic_box_boundaries(), cfg,
                   meta=dict(n_side=n_side, neighbors=neighbors, seed=seed))


def random_box(n_side=12, seed=11, nPerh=1.51, jitter=0.2, vel_scale=0.3, boundaries="periodic", two_lists=False,
               gravity=False):
    """Small irregular test box: jittered lattice, 20% mass noise, random
    velocities and energies, per-node h noise, so every derivative term is
    non-trivial.  boundaries: 'periodic' (all axes), 'reflecting' (walls on
    x, periodic y z) or 'open'.  gravity: add TreeGravity (G = 1, opening
    0.5, softening 0.01; meaningful with open boundaries only)."""
    rng = np.random.default_rng(seed)
    d = 1.0 / n_side
    pos = _lattice(n_side, n_side, n_side, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    n = len(pos)
    pos = pos + rng.normal(0.0, jitter * d, pos.shape)
    if boundaries == "periodic":
        pos = np.mod(pos, 1.0)
    elif boundaries == "reflecting":
        pos[:, 0] = np.clip(pos[:, 0], 1e-9, 1.0 - 1e-9)
        pos[:, 1:] = np.mod(pos[:, 1:], 1.0)
    mass = d ** 3 * (1.0 + 0.2 * rng.uniform(-1.0, 1.0, n))
    rho = 1.0 + 0.1 * rng.uniform(-1.0, 1.0, n)
    eps = 1.5 + 0.5 * rng.uniform(-1.0, 1.0, n)
    vel = rng.normal(0.0, vel_scale, (n, 3))
    h = nPerh * d * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, n))
    if boundaries == "periodic":
        bcs = periodic_box_boundaries()
    elif boundaries == "reflecting":
        bcs = [dict(type=1, axis=0, lo=0.0, hi=1.0, wall_high=0), dict(type=1, axis=0, lo=0.0, hi=1.0, wall_high=1),
               dict(type=0, axis=1, lo=0.0, hi=1.0), dict(type=0, axis=2, lo=0.0, hi=1.0)]
    else:
        bcs = []
    cfg = dict(cfl=0.25, compatible_energy=True, gradh_correction=True, xsph=False, correct_velocity_gradient=True,
               Cl=1.0, Cq=1.0, dt_min=0.0, dt_max=0.1, dt_growth=2.0, last_dt=1.0e-3)
    if gravity:
        cfg.update(gravity=True, G=1.0, softening=0.01, opening=0.5, ftimestep=0.1)
    nodelist = None
    nls = [dict(nPerh=nPerh, hmin=1e-6, hmax=0.5, rhoMin=1e-10, rhoMax=1e10, gamma=GAMMA)]
    if two_lists:
        nodelist = (pos[:, 0] > 0.5).astype(np.int32)
        nls.append(dict(nPerh=nPerh, hmin=1e-6, hmax=0.5, rhoMin=1e-10, rhoMax=1e10, gamma=1.4))
    return Problem("random_box", pos, vel, mass, rho, eps, h, nodelist, nls, bcs, cfg,
                   meta=dict(n_side=n_side, seed=seed, boundaries=boundaries))


def stretched_box(nx=24, ny=18, nz=14, seed=13, nPerh=1.51, jitter=0.15, vel_scale=0.3, tilt=0.15,
                  boundaries="periodic", hminratio=0.1, fix_shape=False):
    """Anisotropic test box for the ASPH smoothing scale: a jittered
    nx x ny x nz lattice in the unit cube (different spacing per axis), with
    H = R diag(1/(nPerh dx), 1/(nPerh dy), 1/(nPerh dz)) R^T rotated per node
    by small random angles (up to ``tilt`` radians) so H carries off-diagonal
    terms, random velocities and energies.  Package settings select
    ASPHClassicSmoothingScale.  boundaries: 'periodic' or 'reflecting'
    (walls on x, periodic y z)."""
    rng = np.random.default_rng(seed)
    d = np.array([1.0 / nx, 1.0 / ny, 1.0 / nz])
    pos = _lattice(nx, ny, nz, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    n = len(pos)
    pos = pos + rng.normal(0.0, 1.0, pos.shape) * (jitter * d)
    if boundaries == "periodic":
        pos = np.mod(pos, 1.0)
        bcs = periodic_box_boundaries()
    else:
        pos[:, 0] = np.clip(pos[:, 0], 1e-9, 1.0 - 1e-9)
        pos[:, 1:] = np.mod(pos[:, 1:], 1.0)
        bcs = [dict(type=1, axis=0, lo=0.0, hi=1.0, wall_high=0), dict(type=1, axis=0, lo=0.0, hi=1.0, wall_high=1),
               dict(type=0, axis=1, lo=0.0, hi=1.0), dict(type=0, axis=2, lo=0.0, hi=1.0)]
    vol = d.prod()
    mass = vol * (1.0 + 0.1 * rng.uniform(-1.0, 1.0, n))
    rho = 1.0 + 0.05 * rng.uniform(-1.0, 1.0, n)
    eps = 1.5 + 0.3 * rng.uniform(-1.0, 1.0, n)
    vel = rng.normal(0.0, vel_scale, (n, 3))
    cfg = dict(cfl=0.25, compatible_energy=True, gradh_correction=True, xsph=False, correct_velocity_gradient=True,
               Cl=1.0, Cq=1.0, dt_min=0.0, dt_max=0.1, dt_growth=2.0, last_dt=1.0e-3,
               smoothing_scale="asph_classic", fix_shape=bool(fix_shape))
    nls = [dict(nPerh=nPerh, hmin=1e-6, hmax=0.5, rhoMin=1e-10, rhoMax=1e10, gamma=GAMMA, hminratio=hminratio)]
    p = Problem("stretched_box", pos, vel, mass, rho, eps, np.full(n, nPerh * d.max()), None, nls, bcs, cfg,
                meta=dict(nx=nx, ny=ny, nz=nz, seed=seed, boundaries=boundaries))
    # per-node rotation R = Rz(c) Ry(b) Rx(a) of the principal axes
    ang = rng.uniform(-tilt, tilt, (n, 3))
    ca, sa = np.cos(ang[:, 0]), np.sin(ang[:, 0])
    cb, sb = np.cos(ang[:, 1]), np.sin(ang[:, 1])
    cc, sc = np.cos(ang[:, 2]), np.sin(ang[:, 2])
    R = np.zeros((n, 3, 3))
    R[:, 0, 0] = cc * cb
    R[:, 0, 1] = cc * sb * sa - sc * ca
    R[:, 0, 2] = cc * sb * ca + sc * sa
    R[:, 1, 0] = sc * cb
    R[:, 1, 1] = sc * sb * sa + cc * ca
    R[:, 1, 2] = sc * sb * ca - cc * sa
    R[:, 2, 0] = -sb
    R[:, 2, 1] = cb * sa
    R[:, 2, 2] = cb * ca
    lam = 1.0 / (nPerh * d) * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, (n, 3)))
    Hm = np.einsum("nik,nk,njk->nij", R, lam, R)
    p.H = np.ascontiguousarray(np.stack([Hm[:, 0, 0], Hm[:, 0, 1], Hm[:, 0, 2], Hm[:, 1, 1], Hm[:, 1, 2],
                                         Hm[:, 2, 2]], axis=1))
    return p


def crksph_box(n_side=10, seed=21, boundaries="periodic", rk_volume="sum", vel_scale=0.3, linear_velocity=None,
               jitter=0.2, two_lists=False):
    """random_box set up for CRKSPH (CRKSPHHydros.py:9-110 defaults): XSPH on,
    LimitedMonaghanGingoldViscosity with Cl = 2 (extent/4) = 1 and
    Cq = (extent/4)^2 = 0.25, no grad-h, compatible energy, IdealH.
    linear_velocity: a 3x3 matrix A to set v = A x (open boundaries)."""
    p = random_box(n_side=n_side, seed=seed, boundaries=boundaries, vel_scale=vel_scale, jitter=jitter,
                   two_lists=two_lists)
    if linear_velocity is not None:
        p.vel = np.ascontiguousarray(p.pos @ np.asarray(linear_velocity, dtype=np.float64).T)
    p.config.update(hydro="crksph", rk_volume=rk_volume, xsph=True, gradh_correction=False,
                    viscosity="limited_monaghan_gingold", Cl=1.0, Cq=0.25, correct_velocity_gradient=False)
    p.name = "crksph_box"
    return p
