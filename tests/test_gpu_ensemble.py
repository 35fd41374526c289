"""Batched ensemble (sphgpu_ensemble_advance): independent boxes of uneven
size advanced concurrently from several host threads, one stream per box.
Every box must end bitwise equal to the same box advanced alone, and a box
that fails must be reported without disturbing the call's return."""
import numpy as np
import pytest

from spheral_gb300 import problems

pytestmark = pytest.mark.gpu

FIELDS = ("position", "velocity", "massDensity", "specificThermalEnergy", "H")


def _boxes():
    sizes = [16, 10, 12, 20, 10, 14, 11]
    return [problems.turbulent_box(s, 40 + k) for k, s in enumerate(sizes)]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("nthreads", [1, 3, 0])
def test_ensemble_equals_single_runs(native_lib, precision, nthreads):
    from spheral_gb300.engine import Engine
    probs = _boxes()
    ens = [Engine.from_problem(p, precision=precision) for p in probs]
    for e in ens:
        e.initialize()
    Engine.ensemble_advance(ens, 4, nthreads=nthreads)
    for p, e in zip(probs, ens):
        ref = Engine.from_problem(p, precision=precision)
        ref.initialize()
        ref.advance(4)
        assert e.time == ref.time
        for f in FIELDS:
            assert np.array_equal(e.field(f), ref.field(f)), (p.meta, f)
        ref.close()
    for e in ens:
        e.close()


def test_ensemble_reports_failing_box(native_lib):
    from spheral_gb300 import _native
    from spheral_gb300.engine import Engine
    probs = _boxes()[:4]
    ens = [Engine.from_problem(p) for p in probs]
    for e in ens:
        e.initialize()
    eps = ens[2].field("specificThermalEnergy")
    eps[5] = np.nan
    ens[2].set_field("specificThermalEnergy", eps)
    with pytest.raises(_native.SphGpuError) as err:
        Engine.ensemble_advance(ens, 3, nthreads=2)
    assert err.value.code == 5
    for e in ens:
        e.close()


def test_ensemble_rejects_repeated_handle(native_lib):
    from spheral_gb300.engine import Engine
    from spheral_gb300 import _native
    e = Engine.from_problem(problems.turbulent_box(10, 1))
    e.initialize()
    L = _native.lib()
    import ctypes
    arr = (ctypes.c_void_p * 2)(e.h, e.h)
    assert L.sphgpu_ensemble_advance(arr, 2, 1, 1e300, 1, None) == 2
    e.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_mixed_method_ensemble_equals_single_runs(native_lib, precision):
    """Boxes with different hydro methods and kernels in one call: CRKSPH
    (summed and mass-over-density volumes, the two-list variant) beside SPH
    boxes with the BSpline and the fifth-order NBSpline tables."""
    from spheral_gb300.engine import Engine
    probs = [problems.crksph_box(12, 3), problems.turbulent_box(12, 7),
             problems.crksph_box(12, 5, rk_volume="mass_over_density"),
             problems.crksph_box(12, 9, two_lists=True)]
    nb = problems.random_box(n_side=16, seed=11, boundaries="periodic")
    nb.config.update(kernel="nbspline", kernel_order=5)
    probs.append(nb)
    ens = [Engine.from_problem(p, precision=precision) for p in probs]
    for e in ens:
        e.initialize()
    Engine.ensemble_advance(ens, 3, nthreads=3)
    for p, e in zip(probs, ens):
        ref = Engine.from_problem(p, precision=precision)
        ref.initialize()
        ref.advance(3)
        assert e.time == ref.time
        for f in FIELDS:
            assert np.array_equal(e.field(f), ref.field(f)), (p.name, f)
        ref.close()
    for e in ens:
        e.close()
