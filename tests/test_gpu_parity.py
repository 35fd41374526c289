"""GPU parity: the sm_103a kernels (called through the C ABI) against the CPU
oracle on identical seeded particles.

Tolerances (FP64 mode):
  * neighbour sets: exact, after mapping oracle ghost nodes to
    (control node, image code);
  * every state and derivative field after one evaluation, and the dt vote:
    normwise relative error <= 1e-12 (summation order differs: the GPU
    gathers per node, the oracle scatters per unordered pair);
  * one full CheapSynchronousRK2 step: <= 1e-11; five steps: <= 1e-9
    (rounding differences are amplified by the step, not by a bug).
"""
import numpy as np
import pytest

from spheral_gb300 import problems

from _parity import DERIV_FIELDS, STATE_FIELDS, compare_fields, ordered_pairs_from_oracle, periodic_axes

pytestmark = pytest.mark.gpu

CASES = {
    "periodic": lambda: problems.random_box(n_side=12, seed=21, boundaries="periodic"),
    "reflecting": lambda: problems.random_box(n_side=12, seed=22, boundaries="reflecting"),
    "open": lambda: problems.random_box(n_side=10, seed=23, boundaries="open"),
    "two_lists": lambda: problems.random_box(n_side=12, seed=24, boundaries="periodic", two_lists=True),
    "sod": lambda: problems.sod(nx1=16, ny1=20),
    "kh": lambda: problems.kelvin_helmholtz(n1=16),
    # low cell occupancy: the neighbour search runs 8- and 16-lane groups
    "sweep_k32": lambda: problems.sweep_box(n_side=24, neighbors=32),
    "sweep_k64": lambda: problems.sweep_box(n_side=20, neighbors=64),
}


def _pair(native_lib, oracle_mod, make, precision="fp64"):
    from spheral_gb300.engine import Engine
    p = make()
    eng = Engine.from_problem(p, precision=precision)
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    return p, eng, orc


@pytest.mark.parametrize("case", list(CASES))
def test_neighbor_sets_exact(native_lib, oracle_mod, case):
    p, eng, orc = _pair(native_lib, oracle_mod, CASES[case])
    i, j, im = eng.pairs()
    got = set(zip(i.tolist(), j.tolist(), im.tolist()))
    assert len(got) == len(i), "duplicate neighbour entries"
    want = ordered_pairs_from_oracle(orc, periodic_axes(p))
    missing, extra = want - got, got - want
    assert not missing and not extra, (sorted(missing)[:10], sorted(extra)[:10])
    assert np.array_equal(eng.field("numNeighbors").astype(np.int64), orc.num_neighbors().astype(np.int64))


@pytest.mark.parametrize("case", list(CASES))
def test_initial_state_parity(native_lib, oracle_mod, case):
    p, eng, orc = _pair(native_lib, oracle_mod, CASES[case])
    bad = compare_fields(eng, orc, STATE_FIELDS, 1e-12)
    assert not bad, bad


@pytest.mark.parametrize("case", list(CASES))
def test_sum_density_parity(native_lib, oracle_mod, case):
    p, eng, orc = _pair(native_lib, oracle_mod, CASES[case])
    eng.sum_density()
    orc.sum_density()
    bad = compare_fields(eng, orc, ["massDensity"], 1e-12, elementwise_tol=1e-12)
    assert not bad, bad


@pytest.mark.parametrize("case", list(CASES))
def test_derivative_parity(native_lib, oracle_mod, case):
    p, eng, orc = _pair(native_lib, oracle_mod, CASES[case])
    eng.evaluate_derivatives()
    orc.evaluate_derivatives()
    bad = compare_fields(eng, orc, DERIV_FIELDS, 1e-12)
    assert not bad, bad


@pytest.mark.parametrize("case", list(CASES))
def test_dt_parity(native_lib, oracle_mod, case):
    p, eng, orc = _pair(native_lib, oracle_mod, CASES[case])
    eng.evaluate_derivatives()
    orc.evaluate_derivatives()
    dg, reason = eng.dt()
    do = orc.hydro_dt()
    assert abs(dg - do) <= 1e-12 * do, (dg, do, reason)


@pytest.mark.parametrize("case", ["periodic", "reflecting", "sod", "kh", "two_lists"])
def test_step_parity(native_lib, oracle_mod, case):
    p, eng, orc = _pair(native_lib, oracle_mod, CASES[case])
    dg = eng.step()
    do = orc.step()
    assert abs(dg - do) <= 1e-12 * do
    bad = compare_fields(eng, orc, STATE_FIELDS, 1e-11)
    assert not bad, bad
    for _ in range(4):
        eng.step()
        orc.step()
    bad = compare_fields(eng, orc, STATE_FIELDS + ["DvDt", "DepsDt", "DvDx"], 1e-9)
    assert not bad, bad
    assert abs(eng.time - orc.time) <= 1e-12 * orc.time


def test_energy_conservation_fp64(native_lib, oracle_mod):
    from spheral_gb300.engine import Engine
    p = problems.random_box(n_side=12, seed=31, boundaries="periodic", vel_scale=0.2)
    eng = Engine.from_problem(p)
    eng.initialize()
    c0 = eng.conservation()
    eng.advance(10)
    c1 = eng.conservation()
    assert abs(c1[7] - c0[7]) <= 1e-12 * abs(c0[7])
    assert abs(c1[0] - c0[0]) <= 1e-14 * c0[0]


def test_deterministic_rerun(native_lib):
    from spheral_gb300.engine import Engine
    p = problems.random_box(n_side=12, seed=41, boundaries="periodic")
    out = []
    for _ in range(2):
        eng = Engine.from_problem(p)
        eng.initialize()
        eng.advance(3)
        out.append(np.concatenate([eng.field(f).ravel() for f in ("position", "velocity", "specificThermalEnergy")]))
        eng.close()
    assert np.array_equal(out[0], out[1])


def test_nonisotropic_H_rejected(native_lib):
    from spheral_gb300 import _native
    from spheral_gb300.engine import Engine
    p = problems.random_box(n_side=12, seed=1)
    p.H[5, 1] = 1e-3
    with pytest.raises(_native.SphGpuError) as e:
        Engine.from_problem(p)
    assert e.value.code == 3


def test_small_periodic_box_rejected(native_lib):
    from spheral_gb300 import _native
    from spheral_gb300.engine import Engine
    p = problems.random_box(n_side=6, seed=1, nPerh=2.0)
    eng = Engine.from_problem(p)
    with pytest.raises(_native.SphGpuError) as e:
        eng.initialize()
    assert e.value.code == 3


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_sod_against_reference_analytic_solution(native_lib, oracle_mod, precision):
    """GPU Sod tube to t = 0.1 against the reference's analytic solution
    (golden fixture) and, in FP64, against the oracle run of the same steps."""
    import os
    from spheral_gb300.engine import Engine
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "sod_analytic.npz"))
    p = problems.sod(nx1=16, ny1=20)
    eng = Engine.from_problem(p, precision=precision)
    eng.initialize()
    steps = 0
    while eng.time < 0.10 - 1e-12:
        eng.step(0.10)
        steps += 1
    x = eng.field("position")[:, 0]
    rho = eng.field("massDensity")
    l1 = float(np.mean(np.abs(rho - np.interp(x, d["x"], d["t0.10_rho"]))))
    assert l1 < 0.02, l1
    if precision == "fp64":
        orc = oracle_mod.Oracle(p)
        orc.initialize()
        for _ in range(steps):
            orc.step(0.10)
        bad = compare_fields(eng, orc, ["position", "velocity", "massDensity", "specificThermalEnergy"], 1e-8)
        assert not bad, bad


def test_nonfinite_state_reported(native_lib):
    """Host-side fault injection: a non-finite specific energy must surface as
    SPHGPU_E_NAN from the step, not as silent propagation."""
    from spheral_gb300 import _native
    from spheral_gb300.engine import Engine
    p = problems.random_box(n_side=12, seed=3)
    eng = Engine.from_problem(p)
    eng.initialize()
    eps = eng.field("specificThermalEnergy")
    eps[17] = np.nan
    eng.set_field("specificThermalEnergy", eps)
    with pytest.raises(_native.SphGpuError) as e:
        eng.step()
        eng.step()
    assert e.value.code == 5


def test_list_capacity_regrows_inside_step(native_lib, oracle_mod):
    """A step whose neighbour counts outgrow the list capacity sized at the
    previous build: the step detects the overflow at its first
    synchronisation, rewrites the lists larger and redoes the sweeps, so the
    lists still equal the oracle's connectivity of the state it started from."""
    from spheral_gb300.engine import Engine
    p = problems.random_box(n_side=12, seed=25, boundaries="open")
    eng = Engine.from_problem(p)
    eng.initialize()
    eng.step()
    st = {f: np.ascontiguousarray(eng.field(f)) for f in
          ("position", "velocity", "mass", "massDensity", "specificThermalEnergy", "H")}
    centre = st["position"].mean(axis=0)
    pos2 = np.ascontiguousarray(centre + 0.6 * (st["position"] - centre))   # ~4.6x the neighbours
    eng.upload_state(pos2, st["velocity"], st["mass"], st["massDensity"], st["specificThermalEnergy"], st["H"])
    eng.step()
    i, j, im = eng.pairs()
    got = set(zip(i.tolist(), j.tolist(), im.tolist()))
    H = st["H"].reshape(-1, 6) if st["H"].ndim == 1 else st["H"]
    p2 = problems.Problem("compressed", pos2, st["velocity"], st["mass"], st["massDensity"],
                          st["specificThermalEnergy"], 1.0 / H[:, 0], None, p.nodelists, [], p.config)
    orc = oracle_mod.Oracle(p2)
    orc.connectivity()
    want = ordered_pairs_from_oracle(orc, ())
    assert got == want
    assert len(got) > 3 * len(p.pos) * 20
