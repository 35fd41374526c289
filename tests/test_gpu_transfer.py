"""Host transfers of the evolved state (sphgpu_upload_state /
sphgpu_download_state): pinned host arrays are read and written in place by
the device in caller order, pageable arrays go through the staged copy.  Both
paths must move the same bits, for isotropic H (expanded to the SymTensor
a I on the way out) and for tensor H (ASPH), and after the internal order has
changed (steps re-sort the nodes)."""
import numpy as np
import pytest

from spheral_gb300 import problems

pytestmark = pytest.mark.gpu

FIELDS = ("position", "velocity", "massDensity", "specificThermalEnergy", "H")


def _pinned(shape):
    torch = pytest.importorskip("torch")
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


def _buffers(n, alloc):
    return [alloc((n, 3)), alloc((n, 3)), alloc(n), alloc(n), alloc((n, 6))]


def _download(eng, alloc):
    b = _buffers(eng.n, alloc)
    for a in b:
        a.fill(np.nan)
    eng.download_state(*b)
    return b


@pytest.mark.parametrize("asph", [False, True])
def test_pinned_and_pageable_transfers_agree(native_lib, asph):
    from spheral_gb300.engine import Engine
    p = problems.stretched_box(seed=141) if asph else problems.random_box(n_side=11, seed=141)
    eng = Engine.from_problem(p, precision="fp32")
    eng.initialize()
    for _ in range(2):
        eng.step()                                   # the internal order differs from the caller's
    pinned = _download(eng, _pinned)
    pageable = _download(eng, lambda s: np.empty(s))
    for a, b, name in zip(pinned, pageable, FIELDS):
        assert np.array_equal(a, b), name
        assert np.array_equal(a.reshape(b.shape), np.asarray(eng.field(name)).reshape(b.shape)), name
    if not asph:
        H = pinned[4]
        assert np.array_equal(H[:, 0], H[:, 3]) and np.array_equal(H[:, 0], H[:, 5])
        assert not H[:, [1, 2, 4]].any()

    # upload a perturbed state through each path into two copies of the engine
    rng = np.random.default_rng(7)
    state = [a.copy() for a in pageable]
    state[0] += 1e-4 * rng.standard_normal(state[0].shape)
    state[1] *= 1.01
    state[3] *= 1.02
    mass = np.asarray(eng.field("mass")).copy()
    image = eng.checkpoint()
    results = []
    for alloc in (_pinned, lambda s: np.empty(s)):
        e = Engine(p.config, precision="fp32")
        for k, nl in enumerate(p.nodelists):
            e.set_nodelist(k, nl["nPerh"], nl["hmin"], nl["hmax"], nl["rhoMin"], nl["rhoMax"], nl["gamma"],
                           nl.get("hminratio"))
        for b in p.boundaries:
            e.add_boundary(b["type"], b["axis"], b["lo"], b["hi"], b.get("wall_high", 0))
        e.restore(image)
        bufs = _buffers(e.n, alloc)
        for dst, src in zip(bufs, state):
            dst[...] = src
        m = alloc(e.n)
        m[...] = mass
        e.upload_state(bufs[0], bufs[1], m, bufs[2], bufs[3], bufs[4])
        got = {f: np.asarray(e.field(f)).copy() for f in FIELDS + ("mass",)}
        e.step()
        got["after"] = np.asarray(e.field("position")).copy()
        results.append(got)
        e.close()
    a, b = results
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["position"].reshape(-1, 3), state[0])
    assert np.array_equal(a["specificThermalEnergy"], state[3])
