"""Domain decomposition on the GPU: the run split into two x-slabs, one
handle per slab (two processes sharing cuda:0, host-staged halos over gloo),
against the same run on one handle.

FP64: the neighbour sets of the owned nodes are exactly those of the single
run (across the cut and the periodic boundary), and after five steps every
state field agrees to 1e-12 normwise (only the summation order of the
neighbour sums differs), as does the dt sequence; the conserved totals (host
sums over the owned nodes) to 1e-11.
Mixed mode: three steps within 5e-5 normwise (the FP32 sweeps see the same
separations relative to different cell origins)."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

from _parity import rel_err

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests"))

pytestmark = pytest.mark.gpu


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run(case, precision, nsteps, world=2):
    import _domain_workers as W
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=W.gpu_rank, args=(r, world, port, case, precision, nsteps, out))
                 for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(300)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        return {k: dict(v) for k, v in out.items()}


def _gather(res, name, n):
    first = res[0][name][1]
    ncomp = len(first[0]) if isinstance(first[0], list) else 1
    out = np.full((n, ncomp), np.nan) if ncomp > 1 else np.full(n, np.nan)
    seen = np.zeros(n, int)
    for r in res.values():
        g, v = r[name]
        out[np.array(g, dtype=np.int64)] = np.array(v)
        seen[np.array(g, dtype=np.int64)] += 1
    assert np.all(seen == 1)
    return out


@pytest.mark.parametrize("case,precision,nsteps,tol", [("box", "fp64", 5, 1e-12), ("walls", "fp64", 5, 1e-12),
                                                        ("kh", "fp64", 3, 1e-12), ("kh", "fp32", 3, 5e-5)])
def test_two_slab_run_matches_single_run(native_lib, case, precision, nsteps, tol):
    import _domain_workers as W
    from spheral_gb300 import problems
    from spheral_gb300.engine import Engine
    res = _run(case, precision, nsteps)
    p = W.make_case(problems, case)
    eng = Engine.from_problem(p, precision=precision)
    eng.initialize()
    if precision == "fp64":
        i, j, _ = eng.pairs()
        want = set(zip(i.tolist(), j.tolist()))
        got = set()
        for r in res.values():
            got |= {tuple(x) for x in r["nbr"]}
        assert got == want, (len(got), len(want), sorted(want - got)[:5], sorted(got - want)[:5])
    dts = [eng.step() for _ in range(nsteps)]
    for r in res.values():
        np.testing.assert_allclose(r["dts"], dts, rtol=1e-12 if precision == "fp64" else 1e-5)
    for name in ("position", "velocity", "massDensity", "specificThermalEnergy", "H"):
        got = _gather(res, name, p.n)
        assert rel_err(got, eng.field(name)) <= tol, (name, rel_err(got, eng.field(name)))
    # totals: host sums over owned nodes against the device tally (summation
    # order differs)
    c = np.array(res[0]["conservation"])
    want_c = eng.conservation()
    assert abs(c[7] - want_c[7]) <= 1e-11 * abs(want_c[7])
    assert abs(c[0] - want_c[0]) <= 1e-12 * abs(want_c[0])
