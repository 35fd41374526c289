"""GPU octree gravity (TreeGravity build + walk) against the oracle's literal
restatement of TreeGravity (per-level hash maps, serial insertion).

Tolerances (FP64 throughout): accelerations and potentials normwise
<= 1e-12 of the oracle (the far/near decisions are taken with the same
expression; only the summation order differs: depth-first pre-order here,
level order in the reference); the gravity time-step vote <= 1e-12; three
full steps of the self-gravitating Evrard problem <= 1e-9.
"""
import numpy as np
import pytest

from spheral_gb300 import problems

from _parity import STATE_FIELDS, compare_fields

pytestmark = pytest.mark.gpu


def _evrard_with_duplicates():
    p = problems.evrard(n=3000, seed=9)
    p.pos[100:140] = p.pos[5] + np.linspace(0.0, 1e-12, 40)[:, None]   # one level-20 leaf with many nodes
    p.pos[200:210] = p.pos[7] + 1e-9
    return p


CASES = {
    "evrard_4096": lambda: problems.evrard(n=4096, seed=2),
    "evrard_20000": lambda: problems.evrard(n=20000, seed=3, opening=0.7),
    "clustered": _evrard_with_duplicates,
    "uniform_box": lambda: problems.random_box(n_side=14, seed=12, boundaries="open", gravity=True),
}


def _gravity_pair(oracle_mod, make, precision="fp64"):
    from spheral_gb300.engine import Engine
    p = make()
    eng = Engine.from_problem(p, precision=precision)
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    eng.evaluate_derivatives()
    orc.evaluate_derivatives()
    orc.gravity()
    return p, eng, orc


@pytest.mark.parametrize("case", list(CASES))
def test_tree_gravity_parity(native_lib, oracle_mod, case):
    p, eng, orc = _gravity_pair(oracle_mod, CASES[case])
    bad = compare_fields(eng, orc, ["DvDtGravity", "potential"], 1e-12)
    assert not bad, bad
    c = eng.conservation()
    assert abs(c[6] - orc.extra_energy()) <= 1e-12 * abs(orc.extra_energy())


@pytest.mark.parametrize("case", ["evrard_4096", "clustered"])
def test_tree_gravity_dt_vote(native_lib, oracle_mod, case):
    p, eng, orc = _gravity_pair(oracle_mod, CASES[case])
    dg, reason = eng.dt()
    # Integrator::selectDt takes the smaller of the hydro vote and TreeGravity's
    # ftimestep * dtMinAcc
    do = min(orc.hydro_dt(), p.config["ftimestep"] * orc.dt_min_acc())
    assert abs(dg - do) <= 1e-12 * do, (dg, do, reason)


@pytest.mark.parametrize("case", ["evrard_20000", "clustered", "uniform_box"])
def test_tree_gravity_in_mixed_mode(native_lib, oracle_mod, case):
    """Mixed walk: FP32 terms on double-float separations with compensated
    sums, FP64 decisions in the guard band.  Same far/near sets as the FP64
    walk, so the only differences are FP32 rounding of each term: normwise
    <= 2e-6 of the oracle (measured ~1e-7)."""
    p, eng, orc = _gravity_pair(oracle_mod, CASES[case], precision="fp32")
    bad = compare_fields(eng, orc, ["DvDtGravity", "potential"], 2e-6)
    assert not bad, bad


def test_evrard_steps_parity(native_lib, oracle_mod):
    from spheral_gb300.engine import Engine
    p = problems.evrard(n=4096, seed=4)
    eng = Engine.from_problem(p)
    orc = oracle_mod.Oracle(p)
    eng.initialize()
    orc.initialize()
    for _ in range(3):
        dg = eng.step()
        do = orc.step()
        assert abs(dg - do) <= 1e-10 * do
    bad = compare_fields(eng, orc, STATE_FIELDS + ["DvDtGravity", "potential"], 1e-9)
    assert not bad, bad
