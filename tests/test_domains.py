"""Host logic of the slab decomposition (spheral_gb300.domains) on gloo CPU
ranks, with an engine double standing in for the GPU handle: ownership and
migration (every node owned by exactly one domain, in the slab it is in,
across the periodic boundary), the halo (exactly the other slabs' nodes
within the halo width, images included), the in-step exchange (every halo
row equals its owner's value at every point) and the all-domain dt minimum."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run(world, nsteps):
    import _domain_workers as W
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=W.double_rank, args=(r, world, port, nsteps, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(150)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        return {k: dict(v) for k, v in out.items()}


@pytest.mark.timeout(200)
@pytest.mark.parametrize("world", [2, 3])
def test_slab_decomposition_routes_every_halo_row(world):
    from spheral_gb300 import problems
    nsteps = 6
    res = _run(world, nsteps)
    p = problems.random_box(n_side=10, seed=5, boundaries="periodic", vel_scale=1.0)
    # every exchange point delivered the owners' values to every halo copy
    for r in range(world):
        assert res[r]["errors"] == [], (r, res[r]["errors"][:5])
    # one dt for all domains, the minimum of their votes
    dts = np.array([res[r]["dts"] for r in range(world)])
    assert np.all(dts == dts[0])
    # ownership: a partition of all nodes; each node where free drift puts it
    gids = np.concatenate([np.array(res[r]["gid"][:res[r]["n_own"]]) for r in range(world)])
    assert np.array_equal(np.sort(gids), np.arange(p.n))
    t = 0.0
    x_expect = p.pos.copy()
    for dt in dts[0]:
        # positions are wrapped between steps; drift since the last wrap
        x_expect = x_expect + p.vel * dt
        t += dt
    L = 1.0
    for r in range(world):
        own = res[r]["n_own"]
        g = np.array(res[r]["gid"][:own])
        pos = np.array(res[r]["pos"])[:own]
        d = pos - x_expect[g]
        d[:, 0] -= L * np.round(d[:, 0] / L)   # the decomposed axis is wrapped between steps
        assert np.max(np.abs(d)) < 1e-12
    # the halo of each domain: exactly the other slabs' nodes within the halo
    # width of its slab at the start of the last step, periodic images included
    xs = {}
    for r in range(world):
        own = res[r]["n_own"]
        for g, x in zip(res[r]["gid"][:own], np.array(res[r]["pos"])[:own, 0]):
            xs[g] = x
    for r in range(world):
        own = res[r]["n_own"]
        hw = res[r]["hwidth"]
        lo, hi = r / world, (r + 1) / world
        last_dt = dts[0][-1]
        want = set()
        for g in range(p.n):
            if g in res[r]["gid"][:own]:
                continue
            x0 = xs[g] - p.vel[g, 0] * last_dt   # where it was when the halo was built
            x0 = np.mod(x0, 1.0)
            for sh in (0.0, 1.0, -1.0):
                xx = x0 + sh
                if max(lo - xx, xx - hi, 0.0) <= hw:
                    want.add((g, sh))
        got = set()
        ghosts = list(zip(res[r]["gid"][own:], np.array(res[r]["pos"])[own:, 0]))
        for g, x in ghosts:
            x0 = x - p.vel[g, 0] * last_dt
            sh = round(x0 - np.mod(x0, 1.0))
            got.add((g, float(sh)))
        assert got == want, (r, sorted(got - want)[:5], sorted(want - got)[:5])
    # some nodes changed domain and some crossed the periodic boundary
    first = set()
    for r in range(world):
        lo, hi = r / world, (r + 1) / world
        first |= {g for g in range(p.n) if lo <= p.pos[g, 0] < hi and g in res[r]["gid"][:res[r]["n_own"]]}
    assert len(first) < p.n
