"""CPU checks of the C-ABI library: it loads, exports every entry point that
include/sphgpu.h declares, builds the kernel table on the host (matching the
oracle's restatement of TableKernel), and fails loudly -- with a status code,
not a crash or a silent fallback -- when no GPU is present."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^\s*(?:int|void|const char\*)\s+(sphgpu_\w+)\s*\(", txt, re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(native_lib):
    names = declared_symbols()
    assert len(names) >= 25
    for n in names:
        assert hasattr(native_lib, n), n


@pytest.mark.parametrize("kernel,order", [("bspline", 3), ("nbspline", 3), ("nbspline", 5), ("nbspline", 7),
                                          ("wendland_c2", 0), ("wendland_c4", 0)])
def test_host_table_matches_oracle(native_lib, oracle_mod, kernel, order):
    from spheral_gb300 import _native, problems
    t = _native.build_kernel_table(1000, kernel, order)
    p = problems.random_box(n_side=12)
    p.config.update(kernel=kernel, kernel_order=order)
    o = oracle_mod.Oracle(p)
    r = o.table()
    for k in ("W", "gradW", "grad2W", "nperh", "wsum", "meta"):
        a, b = t[k], r[k]
        assert a.shape == b.shape
        # bitwise: the quadratic fit amplifies last-bit differences near the kernel edge
        assert np.array_equal(a, b), (k, float(np.max(np.abs(a - b))))


def test_default_config_values(native_lib):
    from spheral_gb300 import _native
    c = _native.default_config()
    assert c.cfl == 0.25 and c.compatible_energy == 1 and c.gradh_correction == 1
    assert c.Cl == 1.0 and c.Cq == 1.0 and c.eps2 == 1.0e-2 and c.num_table_points == 1000


def test_create_without_gpu_fails_loudly(native_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from spheral_gb300 import _native
    c = _native.default_config()
    h = ctypes.c_void_p()
    rc = native_lib.sphgpu_create(ctypes.byref(c), ctypes.byref(h))
    assert rc == 1 and not h.value
    from spheral_gb300.engine import Engine
    with pytest.raises(_native.SphGpuError):
        Engine({})
