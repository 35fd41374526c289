"""Edge cases of the GPU step against the oracle: isolated nodes (no
neighbours: Omega = 1, the isolated-node branch of the IdealH update), a
single node, and a sparse node set spread over a domain whose cell count the
grid has to cap (cells larger than the kernel support only add candidates).

Tolerances as in test_gpu_parity (FP64): fields <= 1e-12 after one
evaluation, five steps <= 1e-9; mixed mode: finite state and exact neighbour
counts."""
import numpy as np
import pytest

from spheral_gb300 import problems

from _parity import DERIV_FIELDS, STATE_FIELDS, compare_fields

pytestmark = pytest.mark.gpu


def _cluster_with_isolated(seed=91, n_side=8, n_iso=6, spread=1.0):
    """A jittered n_side^3 cluster in [0, 1]^3 plus n_iso nodes far from it
    and from one another (open boundaries)."""
    rng = np.random.default_rng(seed)
    d = 1.0 / n_side
    pos = problems._lattice(n_side, n_side, n_side, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    pos = pos + rng.normal(0.0, 0.1 * d, pos.shape)
    iso = np.array([[2.0 + spread * k, -1.5 - 0.7 * k, 0.5 * (-1) ** k] for k in range(n_iso)])
    pos = np.vstack([pos, iso])
    n = len(pos)
    mass = np.full(n, d ** 3) * (1.0 + 0.1 * rng.uniform(-1.0, 1.0, n))
    rho = np.ones(n)
    eps = 1.0 + 0.2 * rng.uniform(-1.0, 1.0, n)
    vel = rng.normal(0.0, 0.1, (n, 3))
    h = np.full(n, 1.51 * d)
    cfg = dict(cfl=0.25, compatible_energy=True, gradh_correction=True, xsph=False, correct_velocity_gradient=True,
               dt_min=0.0, dt_max=0.1, dt_growth=2.0, last_dt=1.0e-3)
    nls = [dict(nPerh=1.51, hmin=1e-6, hmax=0.5, rhoMin=1e-10, rhoMax=1e10, gamma=problems.GAMMA)]
    return problems.Problem("cluster_isolated", pos, vel, mass, rho, eps, h, None, nls, [], cfg)


def _pair(oracle_mod, p, precision="fp64"):
    from spheral_gb300.engine import Engine
    eng = Engine.from_problem(p, precision=precision)
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    return eng, orc


def test_isolated_nodes_parity(native_lib, oracle_mod):
    p = _cluster_with_isolated()
    eng, orc = _pair(oracle_mod, p)
    nn = eng.field("numNeighbors")
    assert (nn[-6:] == 0).all() and (nn[:-6] > 0).all()
    assert np.array_equal(nn.astype(np.int64), orc.num_neighbors().astype(np.int64))
    assert (eng.field("omegaGradh")[-6:] == 1.0).all()
    eng.evaluate_derivatives()
    orc.evaluate_derivatives()
    bad = compare_fields(eng, orc, DERIV_FIELDS, 1e-12)
    assert not bad, bad
    eng2, orc2 = _pair(oracle_mod, _cluster_with_isolated())
    for _ in range(5):
        eng2.step()
        orc2.step()
    bad = compare_fields(eng2, orc2, STATE_FIELDS, 1e-9)
    assert not bad, bad


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_single_node(native_lib, oracle_mod, precision):
    from spheral_gb300.engine import Engine
    p = problems.Problem("one", np.zeros((1, 3)), np.array([[0.1, 0.0, 0.0]]), np.ones(1), np.ones(1),
                         np.ones(1), np.full(1, 0.1), None,
                         [dict(nPerh=1.51, hmin=1e-6, hmax=10.0, rhoMin=1e-10, rhoMax=1e10, gamma=problems.GAMMA)],
                         [], dict(dt_max=0.1, last_dt=1e-3))
    eng = Engine.from_problem(p, precision=precision)
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    for _ in range(3):
        eng.step()
        orc.step()
    assert eng.field("numNeighbors")[0] == 0
    tol = 1e-12 if precision == "fp64" else 1e-5
    bad = compare_fields(eng, orc, ["position", "velocity", "massDensity", "specificThermalEnergy", "H"], tol)
    assert not bad, bad


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_sparse_spread_domain(native_lib, oracle_mod, precision):
    # nodes strewn over a box ~2,500 supports wide: the cell count is capped
    p = _cluster_with_isolated(seed=92, n_side=6, n_iso=40, spread=12.0)
    eng, orc = _pair(oracle_mod, p, precision)
    i, j, im = eng.pairs()
    oi, oj, oim = orc.pairs()
    assert len(i) == 2 * len(oi)
    assert np.array_equal(eng.field("numNeighbors").astype(np.int64), orc.num_neighbors().astype(np.int64))
    for _ in range(3):
        eng.step()
        orc.step()
    tol = 1e-10 if precision == "fp64" else 5e-5
    bad = compare_fields(eng, orc, ["position", "velocity", "massDensity", "specificThermalEnergy"], tol)
    assert not bad, bad
