"""The autotuned choices change speed only, never results.

The mixed-mode step picks, by timing, the neighbour-search group width
(8, 16 or 32 lanes), the pair-kernel variant (register budget, software
pipelining, one / two / four slots per loop iteration) and the batch depth
of the compatible-energy sweep.  With each
choice pinned in turn through the tuning entry points
(sphgpu_set_neighbor_width, sphgpu_set_pair_variant,
sphgpu_set_energy_variant), the neighbour lists -- entry order included,
guard-band candidates too -- and every state field after a few steps are
bitwise the same: the search writes each list in candidate order whatever
the width, and the sweeps sum in list order whatever their batching.

Problems: the Kelvin-Helmholtz box (isotropic H, FP64 and mixed mode; the
pair variants also with the limited Q and under CRKSPH) and a stretched
anisotropic box with reflecting walls (tensor H, mixed mode; search widths
and pair variants)."""
import numpy as np
import pytest

from spheral_gb300 import problems

pytestmark = pytest.mark.gpu

FIELDS = ("position", "velocity", "massDensity", "specificThermalEnergy", "H")


def _run(make, precision, nsteps, width=0, pair=-1, energy=-1):
    from spheral_gb300.engine import Engine
    eng = Engine.from_problem(make(), precision=precision)
    eng.set_neighbor_width(width)
    eng.set_pair_variant(pair)
    eng.set_energy_variant(energy)
    eng.initialize()
    i, j, im = eng.pairs()
    lists = (i.copy(), j.copy(), im.copy())
    for _ in range(nsteps):
        eng.step()
    out = {name: eng.field(name).copy() for name in FIELDS}
    if width:
        assert eng.neighbor_width() == width
    return lists, out


def _same(a, b, what):
    (la, fa), (lb, fb) = a, b
    for x, y in zip(la, lb):
        assert np.array_equal(x, y), ("neighbour lists differ", what)
    for name in FIELDS:
        assert np.array_equal(fa[name], fb[name]), (name, what, float(np.max(np.abs(fa[name] - fb[name]))))


CASES = {
    "kh_fp32": (lambda: problems.kelvin_helmholtz(n1=24), "fp32"),
    "kh_fp64": (lambda: problems.kelvin_helmholtz(n1=24), "fp64"),
    "asph_walls_fp32": (lambda: problems.stretched_box(seed=72, boundaries="reflecting"), "fp32"),
}


@pytest.mark.parametrize("case", list(CASES))
def test_search_width_does_not_change_results(native_lib, case):
    make, precision = CASES[case]
    ref = _run(make, precision, 3, width=32)
    for w in (8, 16):
        _same(ref, _run(make, precision, 3, width=w), f"width {w}")


def _kh_limited():
    p = problems.kelvin_helmholtz(n1=24)
    p.config.update(viscosity="limited_monaghan_gingold", Cl=2.0, Cq=2.0)
    return p


def _kh_crksph():
    p = problems.kelvin_helmholtz(n1=24, smooth=0.025)
    p.config.update(hydro="crksph", rk_volume="sum", xsph=False, gradh_correction=False,
                    viscosity="monaghan_gingold", Cl=1.0, Cq=1.0)
    return p


@pytest.mark.parametrize("make", [lambda: problems.kelvin_helmholtz(n1=24), _kh_limited,
                                  lambda: problems.stretched_box(seed=72, boundaries="reflecting"), _kh_crksph],
                         ids=["mg", "limited_q", "asph_walls", "crksph"])
def test_pair_variant_does_not_change_results(native_lib, make):
    from spheral_gb300.engine import Engine
    _, nv = Engine.from_problem(make(), precision="fp32").pair_variant()
    ref = _run(make, "fp32", 3, width=32, pair=0)
    for v in range(1, nv):
        _same(ref, _run(make, "fp32", 3, width=32, pair=v), f"pair variant {v}")


def test_energy_variant_does_not_change_results(native_lib):
    from spheral_gb300.engine import Engine
    make = lambda: problems.kelvin_helmholtz(n1=24)
    _, nv = Engine.from_problem(make(), precision="fp32").energy_variant()
    ref = _run(make, "fp32", 3, width=32, pair=0, energy=0)
    for v in range(1, nv):
        _same(ref, _run(make, "fp32", 3, width=32, pair=0, energy=v), f"energy variant {v}")


def test_tuning_entry_points_reject_bad_values(native_lib):
    from spheral_gb300._native import SphGpuError as SphError
    from spheral_gb300.engine import Engine
    eng = Engine.from_problem(problems.kelvin_helmholtz(n1=16), precision="fp32")
    for bad in (4, 12, 64, -1):
        with pytest.raises(SphError):
            eng.set_neighbor_width(bad)
    _, nv = eng.energy_variant()
    for bad in (-2, nv):
        with pytest.raises(SphError):
            eng.set_energy_variant(bad)
