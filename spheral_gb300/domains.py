"""Domain decomposition of one SPH run: slabs along one axis, one handle per
domain, halo copies refreshed inside the step.

The reference spreads a problem over MPI ranks with DistributedBoundary
(src/Distributed/DistributedBoundary.cc): every rank owns a set of nodes,
receives ghost copies of the other ranks' nodes within a kernel support of
its own (setControlAndGhostNodes), refreshes the ghost fields whenever the
physics has changed them (applyGhostBoundaries / finalizeGhostBoundary),
and the integrator takes the smallest time-step vote of all ranks
(src/Integrator/Integrator.cc:152-153).  Here:

  * Ownership: equal-width slabs of the global box along `axis`; nodes move
    to the slab they are in between steps (migration).
  * Halo: the owned nodes of other slabs within extent * h_max (the largest
    smoothing scale of all nodes, from an all-reduce) of this slab, with
    periodic images placed at their image positions.  The halo is rebuilt
    every step from the owners' restart-image rows (sphgpu_checkpoint), so a
    halo copy starts the step with every carried field of its owner and
    computes its own node-local updates bitwise as its owner does.
  * In-step exchange (sphgpu_set_domain): the density after the start-of-step
    density sum, the time-step minimum, the mid-step grad-h correction and
    the mid-step accelerations and energy rates -- the fields a neighbour
    sum changes that the halo is read for later in the step.
  * Totals: sums over owned nodes, all-reduced.

Transport is torch.distributed point-to-point on host tensors (gloo, or any
backend with send/recv of CPU tensors); each domain's handle may sit on its
own GPU or share one.  Rows travel as float64 (NodeList ids and global ids
are exact in float64).

A `comm` object supplies rank, size, the all-reduces and the pairwise
exchange; TorchComm wraps a torch.distributed process group.
"""
import numpy as np

from . import _native as N
from .problems import Problem

_HEADER_N_OFFSET = 16   # int64 node count inside an image header


class TorchComm:
    """The collectives the decomposition needs, over torch.distributed."""

    def __init__(self, group=None):
        import torch
        import torch.distributed as dist
        self.torch, self.dist, self.group = torch, dist, group
        self.rank = dist.get_rank(group)
        self.size = dist.get_world_size(group)

    def allreduce(self, values, op):
        t = self.torch.tensor(np.atleast_1d(np.asarray(values, dtype=np.float64)))
        self.dist.all_reduce(t, op={"min": self.dist.ReduceOp.MIN, "max": self.dist.ReduceOp.MAX,
                                    "sum": self.dist.ReduceOp.SUM}[op], group=self.group)
        return t.numpy()

    def alltoall_counts(self, counts):
        """counts[s] = items this rank sends to s; returns items received from each rank."""
        t = self.torch.tensor(np.asarray(counts, dtype=np.int64))
        out = [self.torch.zeros_like(t) for _ in range(self.size)]
        self.dist.all_gather(out, t, group=self.group)
        return np.array([int(o[self.rank]) for o in out], dtype=np.int64)

    def exchange(self, sends, recv_sizes):
        """sends[s]: float64 array for rank s (or None); recv_sizes[s]: the
        number of float64 values to receive from s.  Returns the arrays
        received, by source rank."""
        reqs = []
        recv = [None] * self.size
        for s in range(self.size):
            if s != self.rank and recv_sizes[s] > 0:
                recv[s] = self.torch.empty(int(recv_sizes[s]), dtype=self.torch.float64)
                reqs.append(self.dist.irecv(recv[s], src=self.dist.get_global_rank(self.group, s)
                                            if self.group is not None else s, group=self.group))
        for s in range(self.size):
            if s != self.rank and sends[s] is not None and sends[s].size > 0:
                t = self.torch.from_numpy(np.ascontiguousarray(sends[s], dtype=np.float64))
                reqs.append(self.dist.isend(t, dst=self.dist.get_global_rank(self.group, s)
                                            if self.group is not None else s, group=self.group))
        for r in reqs:
            r.wait()
        return [None if r is None else r.numpy() for r in recv]


def _image_parts(image, header_bytes, nrows):
    n = int(np.frombuffer(image[_HEADER_N_OFFSET:_HEADER_N_OFFSET + 8], dtype=np.int64)[0])
    body = header_bytes + nrows * n * 8
    rows = np.frombuffer(image[header_bytes:body], dtype=np.float64).reshape(nrows, n)
    orig = np.frombuffer(image[body:body + 4 * n], dtype=np.int32)
    lists = np.frombuffer(image[body + 4 * n:body + 8 * n], dtype=np.int32)
    return n, rows, orig, lists


def _image(header, rows, lists):
    """A restart image of rows (nrows x n, caller order = row order)."""
    n = rows.shape[1]
    head = bytearray(header)
    head[_HEADER_N_OFFSET:_HEADER_N_OFFSET + 8] = np.int64(n).tobytes()
    return bytes(head) + np.ascontiguousarray(rows, dtype=np.float64).tobytes() + \
        np.arange(n, dtype=np.int32).tobytes() + np.ascontiguousarray(lists, dtype=np.int32).tobytes()


class SlabDecomposition:
    """One domain of a slab decomposition of `problem` along `axis`.

    Every rank builds the same global Problem (the seeded generator); rank r
    keeps the nodes of slab r and the halo around it.  step() advances the
    whole run by one CheapSynchronousRK2 step (all ranks call it together);
    owned() gives this rank's nodes by global index.  make_engine(problem)
    creates the handle of a domain (default: Engine.from_problem on
    `device`); tests substitute an engine double that speaks the same calls.
    """

    def __init__(self, problem, comm, axis=0, precision="fp64", device=0, make_engine=None):
        self.comm, self.axis = comm, int(axis)
        self.precision, self.device = precision, device
        if problem.config.get("gravity") or problem.config.get("hydro", "sph") != "sph":
            raise NotImplementedError("the decomposition covers the SPH hydro step without gravity")
        self.extent = self._kernel_extent(problem)
        per = [b for b in problem.boundaries if b["type"] == N.BOUNDARY_PERIODIC and b["axis"] == self.axis]
        walls = [b for b in problem.boundaries if b["type"] == N.BOUNDARY_REFLECTING and b["axis"] == self.axis]
        self.periodic = bool(per)
        if per:
            self.lo, self.hi = float(per[0]["lo"]), float(per[0]["hi"])
        elif walls:
            self.lo, self.hi = min(float(b["lo"]) for b in walls), max(float(b["hi"]) for b in walls)
        else:
            x = problem.pos[:, self.axis]
            pad = 1e-9 * max(1.0, float(np.ptp(x)))
            self.lo, self.hi = float(x.min()) - pad, float(x.max()) + pad
        self.length = self.hi - self.lo
        R, r = comm.size, comm.rank
        self.slab_lo = self.lo + self.length * r / R
        self.slab_hi = self.lo + self.length * (r + 1) / R if r < R - 1 else self.hi
        # per-domain boundaries: the decomposed axis is open inside the run;
        # its walls stay with the end slabs and its periods become halo images
        self.local_bcs = []
        for b in problem.boundaries:
            if b["axis"] != self.axis:
                self.local_bcs.append(dict(b))
            elif b["type"] == N.BOUNDARY_REFLECTING:
                if (b.get("wall_high", 0) == 0 and r == 0) or (b.get("wall_high", 0) == 1 and r == R - 1):
                    self.local_bcs.append(dict(b))
        self.template = problem
        self.make_engine = make_engine or self._default_engine
        # owned nodes of the initial state, by global index
        gid = np.arange(problem.n)
        own = self._slab_of(problem.pos[:, self.axis]) == r
        H = problem.H
        rows = dict(pos=problem.pos, vel=problem.vel, mass=problem.mass, rho=problem.rho, eps=problem.eps, H=H,
                    lists=problem.nodelist)
        # initial halo from the global problem (every rank holds it)
        self.hwidth = self._halo_width(1.0 / H[:, 0] if not problem.config.get("smoothing_scale") == "asph_classic"
                                       else self._tensor_hmax(H))
        # this domain's halo: the nodes of every other slab (in rank order)
        # within the halo width of this slab, as the owners select them
        x0 = problem.pos[:, self.axis]
        slab0 = self._slab_of(x0)
        ghost_idx, ghost_shift = [], []
        for s in range(R):
            if s == r:
                continue
            idx, shift = self._halo_for(x0, own_mask=slab0 == s, slab=r)
            ghost_idx.append(idx)
            ghost_shift.append(shift)
        gi = np.concatenate(ghost_idx) if ghost_idx else np.zeros(0, np.int64)
        gs = np.concatenate(ghost_shift) if ghost_shift else np.zeros(0)
        oi = gid[own]
        sel = np.concatenate([oi, gi])
        pos = rows["pos"][sel].copy()
        pos[len(oi):, self.axis] += gs
        local = Problem(problem.name + f"_domain{r}", pos, rows["vel"][sel], rows["mass"][sel], rows["rho"][sel],
                        rows["eps"][sel], 1.0 / H[sel, 0], rows["lists"][sel], problem.nodelists, self.local_bcs,
                        problem.config, meta=dict(problem.meta, domain=r, domains=R))
        local.H = np.ascontiguousarray(H[sel])
        self.engine = self.make_engine(local)
        self.engine.initialize()
        self.n_own = len(oi)
        self.gid = sel.astype(np.int64)
        self.header_bytes, self.row_x, self.nrows = self.engine.image_layout("position")
        self.row_hinv = self.engine.image_layout("H")[1]
        self._fresh = True   # the first step runs on the halo built above
        self._setup_exchange_from_initial(problem, own, gi)

    # -- helpers ----------------------------------------------------------------
    @staticmethod
    def _kernel_extent(problem):
        k = problem.config.get("kernel", "bspline")
        if k in ("wendland_c2", "wendland_c4"):
            return 1.0
        if k == "nbspline":
            return float((int(problem.config.get("kernel_order", 3)) + 1) // 2)
        return 2.0

    @staticmethod
    def _tensor_hmax(H):
        """Largest smoothing scale of each tensor H (1 / smallest eigenvalue)."""
        out = np.empty(len(H))
        for k, h in enumerate(H):
            m = np.array([[h[0], h[1], h[2]], [h[1], h[3], h[4]], [h[2], h[4], h[5]]])
            out[k] = 1.0 / np.linalg.eigvalsh(m)[0]
        return out

    def _default_engine(self, problem):
        from .engine import Engine
        return Engine.from_problem(problem, precision=self.precision, device=self.device)

    def _slab_of(self, x):
        R = self.comm.size
        if self.periodic:
            x = self.lo + np.mod(x - self.lo, self.length)
        s = np.floor((x - self.lo) / self.length * R).astype(np.int64)
        return np.clip(s, 0, R - 1)

    def _slab_bounds(self, s):
        R = self.comm.size
        return self.lo + self.length * s / R, (self.lo + self.length * (s + 1) / R if s < R - 1 else self.hi)

    def _halo_width(self, hmax_local):
        hmax = float(self.comm.allreduce([np.max(hmax_local) if len(hmax_local) else 0.0], "max")[0])
        # the neighbour criterion |x_i - x_j| <= extent max(h_i, h_j), with the
        # neighbour grid's relative slack
        return self.extent * hmax * (1.0 + 1.0e-9)

    def _halo_for(self, x, own_mask, slab):
        """Indices (into x, among own_mask) and axis shifts of the nodes within
        the halo width of slab `slab`, images included.  Order: shifts 0, +L,
        -L, and increasing index within each."""
        lo, hi = self._slab_bounds(slab)
        idx_all = np.nonzero(own_mask)[0]
        xs = x[idx_all]
        out_i, out_s = [], []
        shifts = (0.0, self.length, -self.length) if self.periodic else (0.0,)
        for sh in shifts:
            xx = xs + sh
            d = np.maximum(np.maximum(lo - xx, xx - hi), 0.0)
            m = d <= self.hwidth
            out_i.append(idx_all[m])
            out_s.append(np.full(int(m.sum()), sh))
        return np.concatenate(out_i), np.concatenate(out_s)

    def _setup_exchange_from_initial(self, problem, own, ghost_gid):
        """Send lists for the first step: which owned nodes (caller index)
        each other domain holds as halo copies, in that domain's halo order."""
        R, r = self.comm.size, self.comm.rank
        x = problem.pos[:, self.axis]
        pos_of_gid = {int(g): k for k, g in enumerate(self.gid[:self.n_own])}
        self.send_idx = [None] * R
        for s in range(R):
            if s == r:
                continue
            idx, _ = self._halo_for(x, own_mask=own, slab=s)
            self.send_idx[s] = np.array([pos_of_gid[int(g)] for g in idx], dtype=np.int32)
        counts = [0 if i is None else len(i) for i in self.send_idx]
        self.recv_counts = self.comm.alltoall_counts(counts)
        assert int(self.recv_counts.sum()) == len(self.gid) - self.n_own
        self.engine.set_domain(len(self.gid) - self.n_own, self._exchange)

    # -- the in-step exchange -----------------------------------------------------
    def _exchange(self, point, dt):
        if point == N.EXCHANGE_DT:
            return float(self.comm.allreduce([dt], "min")[0])
        w = self.engine.exchange_width(point)
        sends = [None if idx is None else self.engine.exchange_get(point, idx).ravel() for idx in self.send_idx]
        got = self.comm.exchange(sends, [int(c) * w for c in self.recv_counts])
        blocks = [g.reshape(-1, w) for g in got if g is not None]
        rows = np.concatenate(blocks) if blocks else np.zeros((0, w))
        self.engine.exchange_put(point, rows)
        return None

    # -- migration and the new halo between steps -------------------------------
    def _repartition(self):
        R, r = self.comm.size, self.comm.rank
        image = self.engine.checkpoint()
        header = image[:self.header_bytes]
        n, rows, orig, lists = _image_parts(image, self.header_bytes, self.nrows)
        own = orig < self.n_own
        rows = rows[:, own].copy()
        lists = lists[own].astype(np.float64)
        gids = self.gid[orig[own]].astype(np.float64)
        ax = self.row_x + self.axis
        if self.periodic:
            rows[ax] = self.lo + np.mod(rows[ax] - self.lo, self.length)
        # migration to the slab each node is in now
        dest = self._slab_of(rows[ax])
        payload = np.vstack([rows, lists[None, :], gids[None, :]])   # (nrows + 2) x m
        width = payload.shape[0]
        sends = [None if s == r else payload[:, dest == s].T.ravel() for s in range(R)]
        cnt = self.comm.alltoall_counts([0 if s == r else int(np.sum(dest == s)) for s in range(R)])
        got = self.comm.exchange(sends, [int(c) * width for c in cnt])
        keep = [payload[:, dest == r]] + [g.reshape(-1, width).T for g in got if g is not None]
        mine = np.hstack(keep)
        mine = mine[:, np.argsort(mine[-1], kind="stable")]   # owned nodes in global-index order
        n_own = mine.shape[1]
        # the halo: smoothing scales all-reduced, rows of owned nodes near other slabs
        # the "H" row holds 1/h (isotropic) or the smallest eigenvalue of H
        self.hwidth = self._halo_width(1.0 / mine[self.row_hinv])
        xo = mine[ax]
        all_own = np.ones(n_own, bool)
        self.send_idx = [None] * R
        sends = [None] * R
        for s in range(R):
            if s == r:
                continue
            idx, shift = self._halo_for(xo, all_own, s)
            self.send_idx[s] = idx.astype(np.int32)
            block = mine[:, idx].copy()
            block[ax] += shift
            sends[s] = block.T.ravel()
        self.recv_counts = self.comm.alltoall_counts([0 if i is None else len(i) for i in self.send_idx])
        got = self.comm.exchange(sends, [int(c) * width for c in self.recv_counts])
        ghosts = [g.reshape(-1, width).T for g in got if g is not None]
        allrows = np.hstack([mine] + ghosts) if ghosts else mine
        nr = self.nrows
        self.engine.restore(_image(header, allrows[:nr], allrows[nr].astype(np.int32)))
        self.n_own = n_own
        self.gid = allrows[nr + 1].astype(np.int64)
        self.engine.set_domain(allrows.shape[1] - n_own, self._exchange)

    # -- public ---------------------------------------------------------------------
    def step(self, max_time=1.0e300):
        """One step of the whole run (every domain calls it together)."""
        if not self._fresh:
            self._repartition()
        self._fresh = False
        return self.engine.step(max_time)

    @property
    def time(self):
        return self.engine.time

    def owned(self, name):
        """(global indices, values) of field `name` on this domain's nodes.
        Positions on a periodic decomposed axis are reported inside the box
        (the domains wrap them when nodes migrate, between steps)."""
        f = self.engine.field(name)[:self.n_own]
        if name == "position" and self.periodic:
            f = f.copy()
            f[:, self.axis] = self.lo + np.mod(f[:, self.axis] - self.lo, self.length)
        return self.gid[:self.n_own], f

    def conservation(self):
        """Totals of the whole run (all-reduced): mass, momentum (3),
        kinetic, thermal, 0 (no gravity), total."""
        _, m = self.owned("mass")
        _, v = self.owned("velocity")
        _, e = self.owned("specificThermalEnergy")
        local = [np.sum(m), np.sum(m * v[:, 0]), np.sum(m * v[:, 1]), np.sum(m * v[:, 2]),
                 0.5 * np.sum(m * np.sum(v * v, axis=1)), np.sum(m * e), 0.0]
        out = self.comm.allreduce(local, "sum")
        return np.concatenate([out, [out[4] + out[5] + out[6]]])

    def neighbor_gids(self):
        """Unordered set of (global i, global j) for this domain's owned i."""
        i, j, _ = self.engine.pairs()
        m = i < self.n_own
        return set(zip(self.gid[i[m]].tolist(), self.gid[j[m]].tolist()))

    def close(self):
        self.engine.set_domain(0, None)
        self.engine.close()
