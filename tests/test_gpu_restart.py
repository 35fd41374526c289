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


def test_restore_rejects_other_package_or_kernel(native_lib):
    # an image written by SPH is refused by a CRKSPH handle and the reverse,
    # and one written with the cubic B-spline table by an NBSpline(5) handle
    from spheral_gb300 import _native
    from spheral_gb300.engine import Engine
    p = problems.random_box(n_side=10, seed=4)
    sph = Engine.from_problem(p)
    sph.initialize()
    sph_image = sph.checkpoint()
    crk_p = problems.random_box(n_side=10, seed=4)
    crk_p.config.update(hydro="crksph", rk_volume="sum", gradh_correction=False)
    crk = Engine.from_problem(crk_p)
    crk.initialize()
    crk_image = crk.checkpoint()
    nb_p = problems.random_box(n_side=10, seed=4)
    nb_p.config.update(kernel="nbspline", kernel_order=5)
    nb = Engine.from_problem(nb_p)
    for handle, image in ((crk, sph_image), (sph, crk_image), (nb, sph_image)):
        with pytest.raises(_native.SphGpuError) as err:
            handle.restore(image)
        assert err.value.code == 7
    sph.restore(sph_image)   # its own image still loads


def test_restore_rejects_corrupted_order_and_lists(native_lib):
    # the tail of an image is the caller-order map (n ints) then the NodeList
    # ids (n ints); a map that is not a permutation or an id past the image's
    # NodeLists is refused before anything reaches the device
    from spheral_gb300 import _native
    from spheral_gb300.engine import Engine
    p = problems.random_box(n_side=10, seed=5)
    e = Engine.from_problem(p)
    e.initialize()
    image = bytes(e.checkpoint())
    n = p.n
    orig = np.frombuffer(image[len(image) - 8 * n:len(image) - 4 * n], dtype=np.int32).copy()
    ids = np.frombuffer(image[len(image) - 4 * n:], dtype=np.int32).copy()
    assert sorted(orig.tolist()) == list(range(n)) and np.all(ids == 0)
    dup = orig.copy()
    dup[0] = dup[1]
    bad_order = image[:len(image) - 8 * n] + dup.tobytes() + ids.tobytes()
    far = ids.copy()
    far[3] = 5
    bad_list = image[:len(image) - 4 * n] + far.tobytes()
    for bad in (bad_order, bad_list):
        with pytest.raises(_native.SphGpuError) as err:
            e.restore(bad)
        assert err.value.code == 2
    e.restore(image)
