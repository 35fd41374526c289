"""GPU test of the allocation-free entry point sphgpu_conservation_noalloc.

It serves callers that cannot allocate GPU memory while they run (codes that
lend the library slices of their own pre-allocated device pools); the totals
it computes from caller device arrays must equal those of the handle-based
sphgpu_conservation on the same state, call after call, since every call
reuses the same fixed scratch array inside the library.  The file is named to
be collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entry(native_lib):
    f = native_lib.sphgpu_conservation_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p]
    return f


def test_conservation_noalloc_matches_handle(native_lib):
    import torch
    from spheral_gb300 import problems
    from spheral_gb300.engine import Engine
    p = problems.random_box(n_side=12, seed=8, boundaries="periodic")
    eng = Engine.from_problem(p, precision="fp64")
    eng.initialize()
    eng.advance(2)
    want = eng.conservation()
    mass_h = eng.field("mass")
    vel_h = eng.field("velocity")
    dev = torch.device("cuda", 0)
    mass = torch.tensor(mass_h, dtype=torch.float64, device=dev)
    vel = torch.tensor(vel_h.ravel(), dtype=torch.float64, device=dev)
    eps = torch.tensor(eng.field("specificThermalEnergy"), dtype=torch.float64, device=dev)
    out = torch.empty(8, dtype=torch.float64, device=dev)
    f = _entry(native_lib)
    stream = torch.cuda.current_stream(dev).cuda_stream
    scale_p = float(np.sum(mass_h * np.linalg.norm(vel_h, axis=1)))
    for _ in range(2):   # two calls in a row share the library's scratch array
        out.fill_(np.nan)
        rc = f(mass.data_ptr(), vel.data_ptr(), eps.data_ptr(), None, p.n, out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize(dev)
        got = out.cpu().numpy()
        for k in range(8):
            scale = scale_p if k in (1, 2, 3) else abs(want[k])
            assert abs(got[k] - want[k]) <= 1e-12 * max(scale, 1e-300), (k, got[k], want[k])


def test_conservation_noalloc_with_gravity_potential(native_lib):
    # a self-gravitating box: the potential passed as pot gives the 1/2 sum m phi
    # term and the total of the handle's own tally (TreeGravity's extra energy)
    import torch
    from spheral_gb300 import problems
    from spheral_gb300.engine import Engine
    p = problems.random_box(n_side=10, seed=31, boundaries="open", gravity=True)
    eng = Engine.from_problem(p, precision="fp64")
    eng.initialize()
    eng.advance(2)
    want = eng.conservation()
    assert want[6] != 0.0
    dev = torch.device("cuda", 0)
    mass = torch.tensor(eng.field("mass"), dtype=torch.float64, device=dev)
    vel = torch.tensor(eng.field("velocity").ravel(), dtype=torch.float64, device=dev)
    eps = torch.tensor(eng.field("specificThermalEnergy"), dtype=torch.float64, device=dev)
    pot = torch.tensor(eng.field("potential"), dtype=torch.float64, device=dev)
    out = torch.empty(8, dtype=torch.float64, device=dev)
    f = _entry(native_lib)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for _ in range(2):
        out.fill_(np.nan)
        assert f(mass.data_ptr(), vel.data_ptr(), eps.data_ptr(), pot.data_ptr(), p.n, out.data_ptr(), stream) == 0
        torch.cuda.synchronize(dev)
        got = out.cpu().numpy()
        for k in (0, 4, 5, 6, 7):
            assert abs(got[k] - want[k]) <= 1e-12 * abs(want[k]), (k, got[k], want[k])


def test_conservation_noalloc_rejects_sizes(native_lib):
    import torch
    f = _entry(native_lib)
    dev = torch.device("cuda", 0)
    x = torch.zeros(3, dtype=torch.float64, device=dev)
    out = torch.zeros(8, dtype=torch.float64, device=dev)
    assert f(x.data_ptr(), x.data_ptr(), x.data_ptr(), None, (1 << 26) + 1, out.data_ptr(), None) == 4
    assert f(x.data_ptr(), x.data_ptr(), x.data_ptr(), None, 0, out.data_ptr(), None) == 2
