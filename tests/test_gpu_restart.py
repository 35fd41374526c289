"""Checkpoint / restart (sphgpu_checkpoint, sphgpu_restore): a run stopped
after three steps, written to an image and resumed on a new handle ends
bitwise where the uninterrupted six-step run ends."""
import numpy as np
import pytest

from spheral_gb300 import problems

pytestmark = pytest.mark.gpu

FIELDS = ("position", "velocity", "massDensity", "specificThermalEnergy", "H", "DvDt", "DvDx")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("make", [lambda: problems.random_box(n_side=12, seed=71, boundaries="reflecting"),
                                  lambda: problems.evrard(n=4096, seed=5)], ids=["reflecting", "evrard"])
def test_restart_continues_bitwise(native_lib, precision, make):
    from spheral_gb300.engine import Engine
    p = make()
    a = Engine.from_problem(p, precision=precision)
    a.initialize()
    a.advance(6)
    b = Engine.from_problem(p, precision=precision)
    b.initialize()
    b.advance(3)
    image = b.checkpoint()
    b.close()
    c = Engine.from_problem(p, precision=precision)
    c.restore(image)
    c.advance(3)
    assert c.time == a.time
    for f in FIELDS:
        assert np.array_equal(c.field(f), a.field(f)), f


def test_restore_rejects_foreign_image(native_lib):
    from spheral_gb300 import _native
    from spheral_gb300.engine import Engine
    p = problems.random_box(n_side=10, seed=3)
    e = Engine.from_problem(p)
    e.initialize()
    image = bytearray(e.checkpoint())
    other = Engine.from_problem(p, precision="fp32")
    with pytest.raises(_native.SphGpuError) as err:
        other.restore(bytes(image))
    assert err.value.code == 7
    image[0] = ord("X")
    with pytest.raises(_native.SphGpuError) as err:
        e.restore(bytes(image))
    assert err.value.code == 2
