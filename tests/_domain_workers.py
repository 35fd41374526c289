"""Rank bodies of the domain-decomposition tests (spawned processes).

EngineDouble stands in for a domain's GPU handle on the CPU: it speaks the
calls SlabDecomposition makes (checkpoint/restore images, set_domain,
exchange_get/put, step with the four exchange points) with made-up physics
whose values are known functions of each node's identity, so a test can
check that every halo row arrives from its owner, at every point, in the
right order.  Nodes drift with their velocities and the dt is an all-domain
minimum, so nodes migrate between slabs and across the periodic boundary.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = 120                                   # bytes; node count at offset 16
ROWS = ["x", "y", "z", "vx", "vy", "vz", "mass", "hinv"]
WIDTH = {1: 1, 3: 1, 4: 4}


def expected(mass, cycle, point, k=0):
    """The value an owner computes for a node at an exchange point."""
    return np.sin(mass * 1.0e3 + 0.37 * cycle + 1.3 * point + 0.11 * k)


class EngineDouble:
    def __init__(self, problem):
        p = problem
        self.rows = np.vstack([p.pos.T, p.vel.T, p.mass[None, :], (1.0 / (1.0 / p.H[:, 0]))[None, :]]).copy()
        self.lists = p.nodelist.astype(np.int32).copy()
        self.bcs = p.boundaries
        self.time, self.cycle = 0.0, 0
        self.n_ghost, self.fn = 0, None
        self.errors = []
        self.vals = {}

    @property
    def n(self):
        return self.rows.shape[1]

    def initialize(self):
        pass

    def image_layout(self, field=None):
        row = {"position": 0, "H": 7}.get(field) if field else None
        return HEADER, row, len(ROWS)

    def checkpoint(self):
        head = bytearray(HEADER)
        head[16:24] = np.int64(self.n).tobytes()
        head[32:48] = np.array([self.time, float(self.cycle)]).tobytes()
        return bytes(head) + self.rows.tobytes() + np.arange(self.n, dtype=np.int32).tobytes() + self.lists.tobytes()

    def restore(self, image):
        n = int(np.frombuffer(image[16:24], np.int64)[0])
        self.time, cyc = np.frombuffer(image[32:48], np.float64)
        self.cycle = int(cyc)
        body = HEADER + len(ROWS) * n * 8
        self.rows = np.frombuffer(image[HEADER:body], np.float64).reshape(len(ROWS), n).copy()
        orig = np.frombuffer(image[body:body + 4 * n], np.int32)
        assert np.array_equal(orig, np.arange(n))
        self.lists = np.frombuffer(image[body + 4 * n:], np.int32).copy()

    def set_domain(self, n_ghost, fn):
        self.n_ghost, self.fn = n_ghost, fn

    def exchange_width(self, point):
        return WIDTH[point]

    def exchange_get(self, point, idx):
        idx = np.asarray(idx)
        assert np.all(idx < self.n - self.n_ghost), "a halo row was requested from a halo copy"
        return self.vals[point][idx]

    def exchange_put(self, point, rows):
        rows = np.asarray(rows).reshape(self.n_ghost, WIDTH[point])
        self.vals[point][self.n - self.n_ghost:] = rows

    def step(self, max_time=1.0e300):
        self.cycle += 1
        own = self.n - self.n_ghost
        mass = self.rows[6]
        for point in (1, 2, 3, 4):
            if point == 2:
                local = float(np.min(0.004 + 0.002 * np.abs(np.sin(mass[:own] * 7.0e3)))) if own else 1.0
                dt = self.fn(2, local) if self.fn else local
                continue
            w = WIDTH[point]
            v = np.full((self.n, w), np.nan)
            v[:own] = np.stack([expected(mass[:own], self.cycle, point, k) for k in range(w)], axis=1)
            self.vals[point] = v
            if self.fn:
                self.fn(point, None)
            want = np.stack([expected(mass, self.cycle, point, k) for k in range(w)], axis=1)
            if not np.array_equal(v, want):
                self.errors.append((self.cycle, point, int(np.sum(~(v == want)))))
        self.rows[0:3] += self.rows[3:6] * dt
        self.time += dt
        return dt

    def field(self, name):
        if name == "position":
            return self.rows[0:3].T.copy()
        if name == "mass":
            return self.rows[6].copy()
        raise KeyError(name)

    def close(self):
        pass


def _setup(rank, world, port):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from datetime import timedelta
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=120))
    return dist


def double_rank(rank, world, port, nsteps, out):
    """Run the decomposition over EngineDouble handles; report per-rank data."""
    dist = _setup(rank, world, port)
    from spheral_gb300 import problems
    from spheral_gb300.domains import SlabDecomposition, TorchComm
    p = problems.random_box(n_side=10, seed=5, boundaries="periodic", vel_scale=1.0)
    p.mass = np.arange(1, p.n + 1, dtype=np.float64) * 1.0e-6   # node identity in the mass row
    dom = SlabDecomposition(p, TorchComm(), axis=0, make_engine=EngineDouble)
    dts = []
    for _ in range(nsteps):
        dts.append(dom.step())
    eng = dom.engine
    own = dom.n_own
    out[rank] = dict(gid=dom.gid.tolist(), n_own=own, pos=eng.rows[0:3].T.tolist(), errors=eng.errors, dts=dts,
                     time=eng.time, hwidth=dom.hwidth, mass=eng.rows[6].tolist())
    dist.barrier()
    dist.destroy_process_group()


def gpu_rank(rank, world, port, case, precision, nsteps, out):
    """Run a real decomposition of `case` on cuda:0 (every rank shares it)."""
    dist = _setup(rank, world, port)
    from spheral_gb300 import build
    build.build()
    from spheral_gb300 import problems
    from spheral_gb300.domains import SlabDecomposition, TorchComm
    p = make_case(problems, case)
    dom = SlabDecomposition(p, TorchComm(), axis=0, precision=precision, device=0)
    dom.engine.connectivity()
    nbr = dom.neighbor_gids()
    dts = [dom.step() for _ in range(nsteps)]
    res = dict(dts=dts, time=dom.time, conservation=dom.conservation().tolist(), nbr=sorted(nbr))
    for name in ("position", "velocity", "massDensity", "specificThermalEnergy", "H"):
        g, v = dom.owned(name)
        res[name] = (g.tolist(), np.asarray(v).tolist())
    out[rank] = res
    dom.close()
    dist.barrier()
    dist.destroy_process_group()


def make_case(problems, case):
    if case == "box":
        return problems.random_box(n_side=16, seed=17, boundaries="periodic")
    if case == "kh":
        return problems.kelvin_helmholtz(n1=24)
    if case == "walls":
        return problems.random_box(n_side=16, seed=18, boundaries="reflecting")
    raise ValueError(case)
